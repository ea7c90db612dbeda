// Restarted GMRES on the local AMEn operator, with the Krylov basis, the Hessenberg matrix, the
// Givens rotations and the convergence test kept on the device (reference: cpp/gmres.h:34-161).
// The host reads the stop flag only from the iteration where the previous cycle's convergence rate
// predicts the stop; everything else stays device resident.
#include <cmath>

#include "gmres.cuh"
#include "reduce.cuh"
#include "tc_gemm.cuh"

namespace ttgb {

SplitOut LocalOperator::input_split() const {
  SplitOut o;
  if (lowp && tc && prec == kNoPrec) {
    o.hi = tc->xh.p;
    o.lo = tc->xl.p;
    o.nR = dims.n * dims.R;
    o.ld = tc->ld_r;
  }
  return o;
}

void LocalOperator::apply(const double* x, double* y, bool use_prec, cudaStream_t s,
                          bool presplit, const int* gate) const {
  const double* in = x;
  if (use_prec && prec != kNoPrec) {
    apply_prec(x, wp, s);
    in = wp;
  }
  if (lowp) {
    if (prof_lowp) prof_lowp->begin();
    if (tc) {
      tc->apply(in, y, s, presplit && prec == kNoPrec, gate);
    } else {
      cast(in, xf, size(), s);
      local_product(dims, phi_l32, A32, phi_r32, xf, yf, w1f, w2f, s, 1.0f, 0.0f, spA);
      cast(yf, y, dims.rl * dims.m * dims.RL, s);
    }
    if (prof_lowp)
      prof_lowp->end(local_product_gemm_flops(dims, spA), tc ? ((presplit && prec == kNoPrec) ? 3 : 4) : 5);
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

using red::RT;
using red::block_sum;
constexpr int KC = 8;          // vectors per chunk of the projection's multi-dot
constexpr int kMaxVec = 128;   // basis vectors a cycle may hold (RedWS::cap_vec + 1)

// scalar slots after the Hessenberg data in GmresWS::small
enum ScalSlot : int {
  kRhsNorm = 0,   // ||rhs||
  kResNorm,       // ||r|| at the start of the cycle
  kWNorm2,        // ||w||^2 of the operator output, before orthogonalisation
  kHn,            // H[k+1, k]
  kErr,           // |beta[k+1]| / ||rhs||
  kWpNorm2,       // ||w'||^2 after the first projection
  kHp,            // the norm the finishing pass divides by
  kInv,           // its reciprocal
  kMode,          // 0: one projection kept, 1: second projection, 2: second projection, norm taken directly
  kNumScal = 12
};

struct Layout {   // GmresWS::small
  int iters;
  int64_t H, cs, sn, beta, h1, h2, scal, total;
  explicit Layout(int it) : iters(it) {
    H = 0;
    cs = H + (int64_t)(it + 1) * it;
    sn = cs + it;
    beta = sn + it;
    h1 = beta + it + 1;
    h2 = h1 + it + 1;
    scal = h2 + it + 1;
    total = scal + kNumScal;
  }
};

// ||x|| of the cycle's start vector (also ||rhs|| in the first cycle, where r = rhs) and the
// cycle's start state: H, the rotations and beta cleared, beta[0] = ||r||, the flag words reset.
__global__ void __launch_bounds__(RT) cycle_start_kernel(const double* __restrict__ x, int64_t n,
                                                          int64_t chunk, double* partial,
                                                          unsigned* counter, double* scal,
                                                          int first, int iters, double* H,
                                                          double* cs, double* sn, double* beta,
                                                          int* flag) {
  __shared__ double sh[32];
  const int64_t beg = blockIdx.x * chunk, end = min(n, beg + chunk);
  double s = 0.0;
  for (int64_t i = beg + threadIdx.x; i < end; i += blockDim.x) {
    const double v = x[i];
    s = fma(v, v, s);
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
  if (!red::take_last_ticket(counter)) return;
  const int tid = threadIdx.x;
  for (int i = tid; i < (iters + 1) * iters; i += blockDim.x) H[i] = 0.0;
  for (int i = tid; i < iters; i += blockDim.x) { cs[i] = 0.0; sn[i] = 0.0; }
  for (int i = tid; i < iters + 1; i += blockDim.x) beta[i] = 0.0;
  __syncthreads();
  double tot = 0.0;
  if (tid < 32) tot = red::warp_sum_partials(partial, 0, gridDim.x);
  if (tid == 0) {
    const double nr = sqrt(tot);
    if (first) scal[kRhsNorm] = nr;
    scal[kResNorm] = nr;
    beta[0] = nr;
    flag[kGmresState] = (nr > 0.0) ? 0 : 2;   // 2: r == 0, nothing to do (gmres.h:56-65)
    flag[kGmresBreakdown] = 0;
    flag[kGmresAtIter] = -1;
    flag[kGmresReorth] = 0;
    flag[kGmresReorthVecs] = 0;
  }
  red::reset_ticket(counter);
}

// element i of the operator's next input, also written as its TF32 split when o has a target
__device__ __forceinline__ void put_split(const SplitOut& o, int64_t i, double v) {
  const float f = (float)v;
  const float h = to_tf32(f);
  const int64_t off = (i % o.nR) * o.ld + i / o.nR;
  o.hi[off] = h;
  o.lo[off] = to_tf32(f - h);
}

// y = x / den (den device, y = x when den <= 0); y may alias x
__global__ void scale_by_kernel(const double* x, double* y, int64_t n, const double* den,
                                SplitOut so) {
  const double d = *den;
  const double f = (d > 0.0) ? 1.0 / d : 1.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[i] * f;
    y[i] = v;
    if (so.hi) put_split(so, i, v);
  }
}

// Arnoldi pass 1: h1 = V^T w over the kv basis vectors, and ||w||^2.
__global__ void __launch_bounds__(RT) arnoldi_project_kernel(const double* __restrict__ Q,
                                                              int64_t ldq, int kv,
                                                              const double* __restrict__ w,
                                                              int64_t n, int64_t chunk,
                                                              double* partial, unsigned* counter,
                                                              double* h1, double* scal,
                                                              const int* gate) {
  __shared__ double sh[32];
  __shared__ double shv[(RT / 32) * KC];
  if (*gate != 0) return;   // an iteration queued past the cycle's stopping point
  const int G = gridDim.x;
  const int64_t beg = blockIdx.x * chunk, end = min(n, beg + chunk);
  double ww = 0.0;
  for (int c0 = 0; c0 < kv; c0 += KC) {
    double acc[KC];
#pragma unroll
    for (int j = 0; j < KC; ++j) acc[j] = 0.0;
    const int nc = min(KC, kv - c0);
    for (int64_t i = beg + threadIdx.x; i < end; i += blockDim.x) {
      const double qv = w[i];
      if (c0 == 0) ww = fma(qv, qv, ww);
#pragma unroll
      for (int j = 0; j < KC; ++j)
        if (j < nc) acc[j] = fma(Q[(int64_t)(c0 + j) * ldq + i], qv, acc[j]);
    }
    red::block_sums_to_partials<KC>(acc, nc, shv, partial, c0, G);
  }
  ww = block_sum(ww, sh);
  if (threadIdx.x == 0) partial[(int64_t)kv * G + blockIdx.x] = ww;
  if (!red::take_last_ticket(counter)) return;
  red::reduce_vectors(partial, kv + 1, G, [&](int v, double t) {
    if (v < kv) h1[v] = t;
    else scal[kWNorm2] = t;
  });
  red::reset_ticket(counter);
}

// Arnoldi pass 2: w' = w - V h1 and, in the same pass over V, h2 = V^T w' and ||w'||^2. With
// KB > 0 (kv <= KB) each thread keeps its element's kv basis entries and the kv partial dots in
// registers, so V is read once; KB = 0 re-reads the block's slice of V for the dots. The last block chooses
// the finishing pass (classical Gram-Schmidt with the reorthogonalisation criterion of Daniel,
// Gragg, Kaufman and Stewart, Math. Comp. 30 (1976), with eta = 1/sqrt(2)):
//   mode 0: ||w'||^2 >= ||w||^2 / 2, the first projection is kept, hp = ||w'||;
//   mode 1: w'' = w' - V h2 with ||w''||^2 = ||w'||^2 - ||h2||^2 (V orthonormal), used while the
//           difference keeps at least half of ||w'||^2 (no cancellation to speak of);
//   mode 2: w'' = w' - V h2 with its norm taken from the finished vector (near breakdown).
template <int KB>
__global__ void __launch_bounds__(RT, KB <= 8 ? 2 : 1) arnoldi_reorth_kernel(const double* __restrict__ Q,
                                                             int64_t ldq, int kv,
                                                             const double* __restrict__ h1,
                                                             double* w, int64_t n, int64_t chunk,
                                                             double* partial, unsigned* counter,
                                                             double* h2, double* scal,
                                                             const int* gate, double orth_tol2) {
  __shared__ double sh[32];
  __shared__ double hs[kMaxVec];
  __shared__ double sums[kMaxVec + 1];
  __shared__ double shv[(RT / 32) * (KB > KC ? KB : KC)];
  if (*gate != 0) return;
  const int G = gridDim.x;
  const int64_t beg = blockIdx.x * chunk, end = min(n, beg + chunk);
  for (int j = threadIdx.x; j < kv; j += blockDim.x) hs[j] = h1[j];
  __syncthreads();
  double ss = 0.0;
  if constexpr (KB > 0) {
    double acc[KB];
#pragma unroll
    for (int j = 0; j < KB; ++j) acc[j] = 0.0;
    for (int64_t i = beg + threadIdx.x; i < end; i += blockDim.x) {
      double q[KB];
      double v = w[i];
#pragma unroll
      for (int j = 0; j < KB; ++j) {
        if (j < kv) {
          q[j] = Q[(int64_t)j * ldq + i];
          v = fma(-hs[j], q[j], v);
        }
      }
      w[i] = v;
      ss = fma(v, v, ss);
#pragma unroll
      for (int j = 0; j < KB; ++j)
        if (j < kv) acc[j] = fma(q[j], v, acc[j]);
    }
    red::block_sums_to_partials<(KB > 0 ? KB : 1)>(acc, kv, shv, partial, 0, G);
  } else {
    for (int64_t i = beg + threadIdx.x; i < end; i += blockDim.x) {
      double v = w[i];
      for (int j = 0; j < kv; ++j) v = fma(-hs[j], Q[(int64_t)j * ldq + i], v);
      w[i] = v;
      ss = fma(v, v, ss);
    }
    for (int c0 = 0; c0 < kv; c0 += KC) {   // each thread re-reads only the elements it wrote
      double acc[KC];
#pragma unroll
      for (int j = 0; j < KC; ++j) acc[j] = 0.0;
      const int nc = min(KC, kv - c0);
      for (int64_t i = beg + threadIdx.x; i < end; i += blockDim.x) {
        const double qv = w[i];
#pragma unroll
        for (int j = 0; j < KC; ++j)
          if (j < nc) acc[j] = fma(Q[(int64_t)(c0 + j) * ldq + i], qv, acc[j]);
      }
      red::block_sums_to_partials<KC>(acc, nc, shv, partial, c0, G);
    }
  }
  ss = block_sum(ss, sh);
  if (threadIdx.x == 0) partial[(int64_t)kv * G + blockIdx.x] = ss;
  if (!red::take_last_ticket(counter)) return;
  red::reduce_vectors(partial, kv + 1, G, [&](int v, double t) {
    sums[v] = t;
    if (v < kv) h2[v] = t;
  });
  __syncthreads();
  if (threadIdx.x == 0) {
    const double a = sums[kv], ww = scal[kWNorm2];
    double b = 0.0;
    for (int j = 0; j < kv; ++j) b = fma(sums[j], sums[j], b);
    double mode, hp, inv;
    // b <= orth_tol^2 a: the new vector's component along the basis, |V^T w'| / |w'|, is already
    // below the tolerated loss of orthogonality, so the second projection is not needed either
    if (!(a < 0.5 * ww) || (a > 0.0 && b <= orth_tol2 * a)) {   // NaN: the finishing pass reports it
      mode = 0.0;
      hp = sqrt(a);
      inv = (hp > 0.0) ? 1.0 / hp : 1.0;
    } else if (a > 0.0 && a - b >= 0.5 * a) {
      mode = 1.0;
      hp = sqrt(a - b);
      inv = 1.0 / hp;
    } else {
      mode = 2.0;
      hp = 1.0;
      inv = 1.0;
    }
    scal[kWpNorm2] = a;
    scal[kHp] = hp;
    scal[kInv] = inv;
    scal[kMode] = mode;
  }
  red::reset_ticket(counter);
}

// Arnoldi pass 3: q_{k+1} = (w' - V h2) / hp (mode 1, 2) or w' / hp (mode 0), and its norm nu;
// with a split target, q_{k+1} is also written as the tcgen05 engine's TF32 operand, so the next
// operator application starts from it without a split launch.
// The last block corrects the scale when nu is not 1 to rounding (mode 2, or a cancelled norm),
// then applies the Givens rotations to the new Hessenberg column, takes the new one, and updates
// the residual estimate and the stop flag (apply_givens_rotation_cpu and the convergence test,
// cpp/gmres.h:20-31,105-129). Once the flag is set, later iterations leave H, beta and the flag
// alone, so iterations queued past the stopping point change nothing the solution uses.
__global__ void __launch_bounds__(RT) arnoldi_finish_kernel(
    const double* __restrict__ Q, int64_t ldq, int kv, const double* __restrict__ h1,
    const double* __restrict__ h2, double* w, int64_t n, int64_t chunk, double* partial,
    unsigned* counter, double* scal, int k, int iters, double* H, double* cs, double* sn,
    double* beta, double threshold, int* flag, SplitOut so) {
  __shared__ double sh[32];
  __shared__ double hs[kMaxVec];
  __shared__ double fac;
  if (flag[kGmresState] != 0) return;   // queued past the stopping point: nothing changes
  const int mode = (int)scal[kMode];
  const double inv = scal[kInv];
  if (mode != 0)
    for (int j = threadIdx.x; j < kv; j += blockDim.x) hs[j] = h2[j];
  __syncthreads();
  const int64_t beg = blockIdx.x * chunk, end = min(n, beg + chunk);
  double ss = 0.0;
  for (int64_t i = beg + threadIdx.x; i < end; i += blockDim.x) {
    double v = w[i];
    if (mode != 0)
      for (int j = 0; j < kv; ++j) v = fma(-hs[j], Q[(int64_t)j * ldq + i], v);
    v *= inv;
    w[i] = v;
    if (so.hi) put_split(so, i, v);
    ss = fma(v, v, ss);
  }
  ss = block_sum(ss, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = ss;
  if (!red::take_last_ticket(counter)) return;
  double tot = 0.0;
  if (threadIdx.x < 32) tot = red::warp_sum_partials(partial, 0, gridDim.x);
  if (threadIdx.x == 0) {
    const double nu = sqrt(tot);
    double hn = scal[kHp], f = 1.0;
    if (mode == 2) {
      hn = nu;
      if (nu > 0.0) f = 1.0 / nu;
    } else if (nu > 0.0 && fabs(nu - 1.0) > 1e-10) {
      f = 1.0 / nu;
      hn *= nu;
    }
    fac = f;
    scal[kHn] = hn;
    if (flag[kGmresState] == 0) {
      double* hc = H + (int64_t)k * (iters + 1);
      for (int i = 0; i <= k; ++i) hc[i] = (mode != 0) ? h1[i] + h2[i] : h1[i];
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
      const double err = fabs(beta[k + 1]) / scal[kRhsNorm];
      scal[kErr] = err;
      const bool breakdown = !(hn > 0.0) || !isfinite(hn);
      int state = (err <= threshold || breakdown) ? 1 : 0;
      if (!isfinite(err)) state = 3;
      flag[kGmresState] = state;
      flag[kGmresBreakdown] = breakdown ? 1 : 0;
      if (state != 0) flag[kGmresAtIter] = k;
      if (mode != 0) {
        flag[kGmresReorth] += 1;
        flag[kGmresReorthVecs] += kv;
      }
    }
  }
  __syncthreads();
  if (fac != 1.0) {   // rare: only when the direct norm differs from the divisor used above
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
      const double v = w[i] * fac;
      w[i] = v;
      if (so.hi) put_split(so, i, v);
    }
  }
  red::reset_ticket(counter);
}

// sol += V[:, 0..kk] y (sol = V y when `first`, the start x0 = 0) with
// y = H[0..kk, 0..kk]^{-1} beta[0..kk] (upper triangular after the rotations; gmres.h:131-139).
// Every block solves the small triangular system itself (warp 0, the inner sums across the
// warp), then adds its slice of the combination.
__global__ void __launch_bounds__(RT) cycle_update_kernel(int kk, int iters, const double* H,
                                                           const double* beta,
                                                           const double* __restrict__ Q,
                                                           int64_t ldq, double* sol, int64_t n,
                                                           int first) {
  __shared__ double ys[kMaxVec];
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    for (int i = kk; i >= 0; --i) {
      double t = 0.0;
      for (int j = i + 1 + lane; j <= kk; j += 32) t = fma(H[(int64_t)j * (iters + 1) + i], ys[j], t);
      t = red::warp_sum(t);
      if (lane == 0) {
        const double d = H[(int64_t)i * (iters + 1) + i];
        ys[i] = (d != 0.0) ? (beta[i] - t) / d : 0.0;
      }
      __syncwarp();
    }
  }
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double v = first ? 0.0 : sol[i];
    for (int j = 0; j <= kk; ++j) v = fma(ys[j], Q[(int64_t)j * ldq + i], v);
    sol[i] = v;
  }
}

unsigned elem_grid(int64_t n) {
  unsigned g = cdiv(n, 256);
  const unsigned cap = (unsigned)num_sms() * 8;
  if (g > cap) g = cap;
  if (g == 0) g = 1;
  return g;
}

void launch_reorth(int kv, dim3 g, const double* Q, int64_t ldq, const double* h1, double* w,
                   int64_t n, int64_t chunk, const RedWS& red, double* h2, double* scal,
                   const int* gate, double orth_tol2, cudaStream_t s) {
  if (kv <= 4)
    arnoldi_reorth_kernel<4><<<g, RT, 0, s>>>(Q, ldq, kv, h1, w, n, chunk, red.partial, red.counter, h2, scal, gate, orth_tol2);
  else if (kv <= 8)
    arnoldi_reorth_kernel<8><<<g, RT, 0, s>>>(Q, ldq, kv, h1, w, n, chunk, red.partial, red.counter, h2, scal, gate, orth_tol2);
  else if (kv <= 16)
    arnoldi_reorth_kernel<16><<<g, RT, 0, s>>>(Q, ldq, kv, h1, w, n, chunk, red.partial, red.counter, h2, scal, gate, orth_tol2);
  else
    arnoldi_reorth_kernel<0><<<g, RT, 0, s>>>(Q, ldq, kv, h1, w, n, chunk, red.partial, red.counter, h2, scal, gate, orth_tol2);
  TTGB_CHECK_LAUNCH();
}

}  // namespace

// Iterations of a cycle before its first flag read: the convergence rate of the last converged
// cycle, log(threshold) / iterations, predicts how many this threshold needs; the first read comes
// one iteration before that, and later reads follow every iteration. A stop earlier than predicted
// leaves the iterations queued after it, whose kernels read the flag and return at once; a later
// stop costs one more read per extra iteration.
static int first_read(const GmresWS& ws, double threshold, int iters) {
  if (!(ws.log_rate < 0.0) || !(threshold > 0.0) || !(threshold < 1.0)) return 1;
  const double need = std::log(threshold) / ws.log_rate;
  if (!(need < (double)iters)) return iters;
  int p = (int)std::ceil(need) - 1;
  return p < 1 ? 1 : p;
}

GmresResult gmres(const LocalOperator& op, const double* rhs, double* sol, int iters,
                  double threshold, int resets, GmresWS& ws, const RedWS& red, cudaStream_t s,
                  double orth_tol) {
  GmresResult res;
  const int64_t n = op.size();
  TTGB_REQUIRE(iters >= 1, "gmres: local_iterations must be >= 1");
  TTGB_REQUIRE(iters + 1 <= red.cap_vec && iters + 1 <= kMaxVec,
               "gmres: local_iterations exceeds the Krylov workspace (at most 126)");
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
  double* scal = sm + L.scal;
  int G1; int64_t ch1;
  red_launch_dims(red, n, 1, G1, ch1);
  // the kernels that write the operator's next input also write its tcgen05 operand split
  const SplitOut so = op.input_split();

  // x0 = 0: the first cycle's update writes sol, so it is not cleared beforehand
  for (int cycle = 0; cycle < resets; ++cycle) {
    // r = rhs - op(sol) into Q_0, ||r||, the cycle's start state, Q_0 = r / ||r||
    const double* r = rhs;
    if (cycle > 0) {
      op.apply(sol, Q, true, s);
      sub(rhs, Q, Q, n, s);
      r = Q;
    }
    cycle_start_kernel<<<G1, RT, 0, s>>>(r, n, ch1, red.partial, red.counter, scal, cycle == 0 ? 1 : 0,
                                         iters, H, cs, sn, beta, ws.d_flag);
    TTGB_CHECK_LAUNCH();
    scale_by_kernel<<<elem_grid(n), 256, 0, s>>>(r, Q, n, &scal[kResNorm], so);
    TTGB_CHECK_LAUNCH();
    const int first = first_read(ws, threshold, iters);
    int k = 0;
    int state = 0;
    for (k = 0; k < iters; ++k) {
      const int kv = k + 1;
      double* qk = Q + (int64_t)k * n;
      double* w = Q + (int64_t)kv * n;
      // q_k's split was written with q_k; past the stopping point the product does nothing
      op.apply(qk, w, true, s, so.hi != nullptr, ws.d_flag + kGmresState);
      if (op.prof_krylov) op.prof_krylov->begin();
      int G; int64_t chunk;
      red_launch_dims(red, n, kv + 1, G, chunk);
      arnoldi_project_kernel<<<G, RT, 0, s>>>(Q, n, kv, w, n, chunk, red.partial, red.counter, h1, scal,
                                              ws.d_flag + kGmresState);
      TTGB_CHECK_LAUNCH();
      launch_reorth(kv, dim3(G), Q, n, h1, w, n, chunk, red, h2, scal, ws.d_flag + kGmresState,
                    orth_tol * orth_tol, s);
      arnoldi_finish_kernel<<<G, RT, 0, s>>>(Q, n, kv, h1, h2, w, n, chunk, red.partial, red.counter,
                                             scal, k, iters, H, cs, sn, beta, threshold, ws.d_flag,
                                             so);
      TTGB_CHECK_LAUNCH();
      // bytes of the reference's MGS iteration, 8 N (2k + 3), and of the three passes here
      // without the second projection, 8 N (2k + 7); the second projection's kv reads are added
      // per cycle from the device's count
      if (op.prof_krylov)
        op.prof_krylov->end(8.0 * (double)n * (2 * k + 3), 3, 8.0 * (double)n * (2 * k + 7));
      if (k + 1 >= first || k == iters - 1) {
        TTGB_CUDA(cudaMemcpyAsync(ws.h_flag, ws.d_flag, kGmresFlagWords * sizeof(int),
                                  cudaMemcpyDeviceToHost, s));
        TTGB_CUDA(cudaStreamSynchronize(s));
        ++res.syncs;
        state = ws.h_flag[kGmresState];
        if (state != 0) break;
      }
    }
    if (state == 2) {          // nothing to do in this cycle (gmres.h:56-65)
      if (cycle == 0) fill(sol, 0.0, n, s);
      res.flag = 1;
      res.overrun += (k < iters ? k : iters - 1) + 1;
      break;
    }
    if (state == 3) throw Error(kNumericalError, "GMRES: non-finite residual");
    const int kk = (state == 1) ? ws.h_flag[kGmresAtIter] : iters - 1;   // gmres.h:131
    res.overrun += (k < iters ? k : iters - 1) - kk;
    res.reorth += ws.h_flag[kGmresReorth];
    if (op.prof_krylov) op.prof_krylov->aux += 8.0 * (double)n * ws.h_flag[kGmresReorthVecs];
    cycle_update_kernel<<<elem_grid(n), RT, 0, s>>>(kk, iters, H, beta, Q, n, sol, n,
                                                    cycle == 0 ? 1 : 0);
    TTGB_CHECK_LAUNCH();
    res.nit += kk + 1;
    if (state == 1) {
      if (threshold > 0.0 && threshold < 1.0) ws.log_rate = std::log(threshold) / (kk + 1);
      res.flag = 1;
      break;
    }
    ws.log_rate = 0.0;   // no converged cycle to predict from: read every iteration next time
  }
  return res;
}

}  // namespace ttgb
