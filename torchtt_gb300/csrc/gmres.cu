// Restarted GMRES on the local AMEn operator, with the Krylov basis, the Hessenberg matrix, the
// Givens rotations and the convergence test kept on the device (reference: cpp/gmres.h:34-161).
// The host reads one 8-byte flag per iteration to stop; everything else stays device resident.
#include <cmath>

#include "gmres.cuh"

namespace ttgb {

void LocalOperator::apply(const double* x, double* y, bool use_prec, cudaStream_t s) const {
  const double* in = x;
  if (use_prec && prec != kNoPrec) {
    apply_prec(x, wp, s);
    in = wp;
  }
  if (lowp) {
    if (prof_lowp) prof_lowp->begin();
    if (tc) {
      tc->apply(in, y, s);
    } else {
      cast(in, xf, size(), s);
      local_product(dims, phi_l32, A32, phi_r32, xf, yf, w1f, w2f, s, 1.0f, 0.0f, spA);
      cast(yf, y, dims.rl * dims.m * dims.RL, s);
    }
    if (prof_lowp) prof_lowp->end(local_product_gemm_flops(dims, spA), tc ? 4 : 5);
    if (count_lowp) ++*count_lowp;
    return;
  }
  Fp64EngineScope eng(fp64_engine);
  if (prof) prof->begin();
  local_product(dims, phi_l, A, phi_r, in, y, w1, w2, s, 1.0, 0.0, spA);
  if (prof) prof->end(local_product_gemm_flops(dims, spA), 3);
  if (count) ++*count;
}

void LocalOperator::apply_fp64(const double* x, double* y, cudaStream_t s) const {
  Fp64EngineScope eng(fp64_engine);
  if (prof) prof->begin();
  local_product(dims, phi_l, A, phi_r, x, y, w1, w2, s, 1.0, 0.0, spA);
  if (prof) prof->end(local_product_gemm_flops(dims, spA), 3);
  if (count) ++*count;
}

namespace {

// layout of GmresWS::small
struct Layout {
  int iters;
  int64_t H, cs, sn, beta, h1, h2, y, scal, total;
  explicit Layout(int it) : iters(it) {
    H = 0;
    cs = H + (int64_t)(it + 1) * it;
    sn = cs + it;
    beta = sn + it;
    h1 = beta + it + 1;
    h2 = h1 + it + 1;
    y = h2 + it + 1;
    scal = y + it + 1;
    total = scal + 8;
  }
};

__global__ void gmres_start_kernel(double* beta, double* scal, int iters, double* H, double* cs,
                                   double* sn, int* flag) {
  // scal[0] = ||rhs||, scal[1] = ||r||
  const int tid = threadIdx.x;
  for (int i = tid; i < (iters + 1) * iters; i += blockDim.x) H[i] = 0.0;
  for (int i = tid; i < iters; i += blockDim.x) { cs[i] = 0.0; sn[i] = 0.0; }
  for (int i = tid; i < iters + 1; i += blockDim.x) beta[i] = 0.0;
  __syncthreads();
  if (tid == 0) {
    beta[0] = scal[1];
    flag[0] = (scal[1] > 0.0) ? 0 : 2;   // 2: r == 0, nothing to do (gmres.h:56-65)
    flag[1] = 0;
  }
}

__global__ void gmres_step_kernel(int k, int iters, const double* h1, const double* h2,
                                  double* scal, double* H, double* cs, double* sn, double* beta,
                                  double threshold, int* flag) {
  if (threadIdx.x != 0) return;
  if (flag[0] == 2) return;   // the cycle started from a zero residual
  double* hc = H + (int64_t)k * (iters + 1);
  for (int i = 0; i <= k; ++i) hc[i] = h1[i] + h2[i];
  const double hn = sqrt(fmax(scal[2], 0.0));
  scal[3] = hn;
  hc[k + 1] = hn;
  for (int i = 0; i < k; ++i) {   // apply_givens_rotation_cpu, gmres.h:20-31
    const double t = cs[i] * hc[i] + sn[i] * hc[i + 1];
    hc[i + 1] = -sn[i] * hc[i] + cs[i] * hc[i + 1];
    hc[i] = t;
  }
  const double den = sqrt(hc[k] * hc[k] + hc[k + 1] * hc[k + 1]);
  double c = 1.0, s = 0.0;
  if (den > 0.0) { c = hc[k] / den; s = hc[k + 1] / den; }
  hc[k] = c * hc[k] + s * hc[k + 1];
  hc[k + 1] = 0.0;
  cs[k] = c;
  sn[k] = s;
  beta[k + 1] = -s * beta[k];
  beta[k] = c * beta[k];
  const double err = fabs(beta[k + 1]) / scal[0];
  scal[4] = err;
  const bool breakdown = !(hn > 0.0) || !isfinite(hn);
  flag[0] = (err <= threshold || breakdown) ? 1 : 0;
  flag[1] = breakdown ? 1 : 0;
  if (!isfinite(err)) flag[0] = 3;
}

// y = H[0..kk,0..kk]^{-1} beta[0..kk] (upper triangular after the rotations)
__global__ void gmres_backsolve_kernel(int kk, int iters, const double* H, const double* beta,
                                       double* y) {
  if (threadIdx.x != 0) return;
  for (int i = kk; i >= 0; --i) {
    double v = beta[i];
    for (int j = i + 1; j <= kk; ++j) v -= H[(int64_t)j * (iters + 1) + i] * y[j];
    const double d = H[(int64_t)i * (iters + 1) + i];
    y[i] = (d != 0.0) ? v / d : 0.0;
  }
}

}  // namespace

GmresResult gmres(const LocalOperator& op, const double* rhs, double* sol, int iters,
                  double threshold, int resets, GmresWS& ws, const RedWS& red, cudaStream_t s) {
  GmresResult res;
  const int64_t n = op.size();
  TTGB_REQUIRE(iters >= 1, "gmres: local_iterations must be >= 1");
  ws.Q.ensure((size_t)(iters + 1) * n, s);
  Layout L(iters);
  ws.small.ensure((size_t)L.total, s);
  double* Q = ws.Q.p;
  double* sm = ws.small.p;
  double* H = sm + L.H;
  double* cs = sm + L.cs;
  double* sn = sm + L.sn;
  double* beta = sm + L.beta;
  double* h1 = sm + L.h1;
  double* h2 = sm + L.h2;
  double* y = sm + L.y;
  double* scal = sm + L.scal;

  fill(sol, 0.0, n, s);
  nrm2(red, rhs, n, &scal[0], s);
  for (int cycle = 0; cycle < resets; ++cycle) {
    // r = rhs - op(sol) into Q_0
    if (cycle == 0) {
      copy(rhs, Q, n, s);                       // x0 = 0: r = rhs exactly
    } else {
      op.apply(sol, Q, true, s);
      sub(rhs, Q, Q, n, s);
    }
    nrm2(red, Q, n, &scal[1], s);
    gmres_start_kernel<<<1, 256, 0, s>>>(beta, scal, iters, H, cs, sn, ws.d_flag);
    TTGB_CHECK_LAUNCH();
    scale_dev(Q, n, nullptr, &scal[1], s);      // Q_0 = r / ||r||
    int k = 0;
    int flag = 0;
    for (k = 0; k < iters; ++k) {
      double* qk = Q + (int64_t)k * n;
      double* w = Q + (int64_t)(k + 1) * n;
      op.apply(qk, w, true, s);
      if (op.prof_krylov) op.prof_krylov->begin();
      multidot(red, Q, n, k + 1, w, n, h1, s);
      gs_update(red, Q, n, k + 1, h1, w, n, h2, true, false, s);
      gs_update(red, Q, n, k + 1, h2, w, n, &scal[2], false, true, s);
      if (op.prof_krylov)
        op.prof_krylov->end(8.0 * (double)n * (2 * k + 3), 3, 8.0 * (double)n * (4 * k + 10));
      gmres_step_kernel<<<1, 32, 0, s>>>(k, iters, h1, h2, scal, H, cs, sn, beta, threshold,
                                         ws.d_flag);
      TTGB_CHECK_LAUNCH();
      scale_dev(w, n, nullptr, &scal[3], s);
      TTGB_CUDA(cudaMemcpyAsync(ws.h_flag, ws.d_flag, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
      TTGB_CUDA(cudaStreamSynchronize(s));
      flag = ws.h_flag[0];
      if (flag == 2) break;   // initial residual was zero
      if (flag == 3) throw Error(kNumericalError, "GMRES: non-finite residual");
      if (flag == 1) break;
    }
    if (flag == 2) {          // nothing to do in this cycle (gmres.h:56-65)
      res.flag = 1;
      break;
    }
    const int kk = (k < iters) ? k : iters - 1;   // gmres.h:131
    gmres_backsolve_kernel<<<1, 32, 0, s>>>(kk, iters, H, beta, y);
    TTGB_CHECK_LAUNCH();
    combine(Q, n, kk + 1, y, sol, sol, n, s);
    res.nit += kk + 1;
    if (flag == 1) {
      res.flag = 1;
      break;
    }
  }
  return res;
}

}  // namespace ttgb
