// Local AMEn product on tcgen05 (see tc_local.cuh). Every tensor-core operand is stored K-major
// with its rows padded to tc_ld(K) floats (a multiple of 16 bytes), the row pitch the TMA tensor
// maps of tc_gemm need; the padding columns are never read (the copies stop at K).
#include "tc_local.cuh"

namespace ttgb {

void TcCore::build(const double* A, int64_t s, int64_t m, int64_t n, int64_t S, cudaStream_t st) {
  ld = tc_ld(s * n);
  const size_t ne = (size_t)(m * S * ld);
  hi.ensure(ne, st);
  lo.ensure(ne, st);
  Gather4 g;   // A'[m][S][s][n] = A[s][m][n][S], rows (m, S) of s n elements
  g.e0 = n; g.s0 = S;
  g.e1 = s; g.s1 = m * n * S;
  g.e2 = S; g.s2 = 1;
  g.e3 = m; g.s3 = n * S;
  split_tf32(A, g, hi.p, lo.p, st, s * n, ld);
}

void TcLocal::setup(const LocalOpDims& dims, const double* phi_l, const double* phi_r,
                    const TcCore* c, const SparseCore* spa, int* errflag, cudaStream_t st) {
  d = dims;
  core = c;
  sp = (spa && spa->use) ? spa : nullptr;
  err = errflag;
  ld_r = tc_ld(d.r);
  ld_sn = tc_ld(d.s * d.n);
  ld_SR = tc_ld(d.S * d.R);
  phl_h.ensure((size_t)(d.rl * d.s * ld_r), st); phl_l.ensure((size_t)(d.rl * d.s * ld_r), st);
  phr_h.ensure((size_t)(d.RL * ld_SR), st); phr_l.ensure((size_t)(d.RL * ld_SR), st);
  Gather4 g;   // Phi_l[(l, s), r]: rows of r
  g.e0 = d.r; g.s0 = 1;
  g.e1 = d.rl * d.s; g.s1 = d.r;
  split_tf32(phi_l, g, phl_h.p, phl_l.p, st, d.r, ld_r);
  g.e0 = d.S * d.R; g.s0 = 1;   // Phi_r[L, (S, R)]: rows of S R
  g.e1 = d.RL; g.s1 = d.S * d.R;
  split_tf32(phi_r, g, phr_h.p, phr_l.p, st, d.S * d.R, ld_SR);
  const size_t nx = (size_t)(d.n * d.R * ld_r);
  const size_t nw = (size_t)(d.rl * d.R * ld_sn), ny = (size_t)(d.rl * d.m * ld_SR);
  xh.ensure(nx, st); xl.ensure(nx, st);
  if (sp) wf.ensure((size_t)(d.rl * d.s * d.n * d.R), st);
  else { wh.ensure(nw, st); wl.ensure(nw, st); }
  yh.ensure(ny, st); yl.ensure(ny, st);
}

void TcLocal::apply(const double* x, double* y, cudaStream_t st, bool presplit, const int* gate) {
  if (!presplit) {   // x^P[(n,R), r] = x[r, n, R], rows of r
    Gather4 g;
    g.e0 = d.r; g.s0 = d.n * d.R;
    g.e1 = 1;   g.s1 = 0;
    g.e2 = d.R; g.s2 = 1;
    g.e3 = d.n; g.s3 = d.R;
    split_tf32(x, g, xh.p, xl.p, st, d.r, ld_r);
  }
  if (sp) {
    {   // W[l][s][n][R] = x^P[(n,R), r] . Phi_l[(l,s), r]   (FP32)
      TcGemm t;
      t.M = (int)(d.n * d.R); t.N = (int)(d.rl * d.s); t.K = (int)d.r;
      t.A_hi = xh.p; t.A_lo = xl.p; t.lda = ld_r;
      t.B_hi = phl_h.p; t.B_lo = phl_l.p; t.ldb = ld_r;
      t.out = kTcOutF32; t.C32 = wf.p;
      t.cm.e0 = (int)d.R; t.cm.s0 = 1; t.cm.s1 = d.R;                          // row (n, R)
      t.cn.e0 = (int)d.s; t.cn.s0 = d.n * d.R; t.cn.s1 = d.s * d.n * d.R;      // col (l, s)
      t.gate = gate;
      tc_gemm(t, err, st);
    }
    // Y2[l][m][(S, R)] = sum A[s,m,n,S] W[l][s][n][R], written as the TF32 split with rows (l, m)
    // of pitch ld_SR: key (m, S) -> m ld_SR + S R
    StageDims g{d.rl, d.R, d.s * d.n * d.R, d.m * ld_SR, d.R, d.n * d.R, d.R};
    g.ke0 = d.S;
    g.sk1 = ld_SR;
    g.gate = gate;
    sparse_stage_split(sp->lp, wf.p, yh.p, yl.p, g, st);
  } else {
    {   // W[l][R][(s, n)] = x^P[(n,R), r] . Phi_l[(l,s), r], rows (l, R) of pitch ld_sn
      TcGemm t;
      t.M = (int)(d.n * d.R); t.N = (int)(d.rl * d.s); t.K = (int)d.r;
      t.A_hi = xh.p; t.A_lo = xl.p; t.lda = ld_r;
      t.B_hi = phl_h.p; t.B_lo = phl_l.p; t.ldb = ld_r;
      t.out = kTcOutSplit; t.C_hi = wh.p; t.C_lo = wl.p;
      t.cm.e0 = (int)d.R; t.cm.s1 = 1; t.cm.s0 = ld_sn;                     // row (n, R)
      t.cn.e0 = (int)d.s; t.cn.s1 = d.R * ld_sn; t.cn.s0 = d.n;             // col (l, s)
      t.gate = gate;
      tc_gemm(t, err, st);
    }
    {   // Y2_l[(m,S), R] = A'[(m,S),(s,n)] . W_l[R, (s,n)]   (batched over l)
      TcGemm t;
      t.M = (int)(d.m * d.S); t.N = (int)d.R; t.K = (int)(d.s * d.n); t.batch = (int)d.rl;
      t.A_hi = core->hi.p; t.A_lo = core->lo.p; t.lda = core->ld; t.a_bs = 0;
      t.B_hi = wh.p; t.B_lo = wl.p; t.ldb = ld_sn; t.b_bs = d.R * ld_sn;
      t.out = kTcOutSplit; t.C_hi = yh.p; t.C_lo = yl.p;
      t.cm.e0 = (int)d.S; t.cm.s1 = ld_SR; t.cm.s0 = d.R;                   // row (m, S)
      t.cn.s0 = 1; t.c_bs = d.m * ld_SR;
      t.gate = gate;
      tc_gemm(t, err, st);
    }
  }
  {   // y[(l,m), L] = Y2[(l,m),(S,R)] . Phi_r[L,(S,R)]
    TcGemm t;
    t.M = (int)(d.rl * d.m); t.N = (int)d.RL; t.K = (int)(d.S * d.R);
    t.A_hi = yh.p; t.A_lo = yl.p; t.lda = ld_SR;
    t.B_hi = phr_h.p; t.B_lo = phr_l.p; t.ldb = ld_SR;
    t.out = kTcOutF64; t.C64 = y;
    t.cm.s0 = d.RL; t.cn.s0 = 1;
    t.gate = gate;
    tc_gemm(t, err, st);
  }
}

}  // namespace ttgb
