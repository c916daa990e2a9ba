// clbm_adjoint.cu -- discrete adjoint of the interval-integrated drag.
//
// Forward (as in clbm_step.cu): P_0 = C(S_0); for t = 0..T-1:
// S_{t+1} = Pull(P_t), F_t = D(S_{t+1}), P_{t+1} = C(S_{t+1});
// J = kappa * sum_t D(S_{t+1}), kappa = dt * force_scale (the weight
// integral s of src/mpi_LBM_GK_pops_perturb.cpp:445-465; the constant shift
// has no gradient).  Adjoint, sigma_t = dJ/dS_t:
//   sigma_T = kappa grad D(S_T)
//   sigma_t = J_C(S_t)^T Pull^T sigma_{t+1} + kappa grad D(S_t),  1 <= t < T
//   sigma_0 = J_C(S_0)^T Pull^T sigma_1
// Pull^T is a gather too: P(m,k) is read by exactly one slot, the node's own
// (m, opp k) when that slot is bounced back, else (m + c_k, k); square-interior
// nodes carry no sensitivity (they are reset every step).  The collision
// Jacobian is a rank-3 update of (1-omega) I through rho, jx, jy, so its
// transpose costs three reductions per node.  D is the stress-integration drag
// (src/lbm_src/force.cpp:8-144) with Pi_xx^neq = sum_{cx!=0} f - rho/3 - jx^2/rho
// and Pi_xy^neq = f5 - f6 + f7 - f8 - jx jy / rho (its closed form), or under
// drag_mode 1 the momentum exchange, linear in S: -2 c_kx on every slot the
// square bounces back.
#include "clbm_internal.h"
#include "clbm_physics.cuh"

namespace clbm {

template <bool F64>
using real_t = typename std::conditional<F64, double, float>::type;

struct AdjArgs {
  const RunDev *runs;
  int nruns;
  const void *sigma_in;  // sigma_{t+1}
  void *sigma_out;       // sigma_t
  const void *P;         // P_{t-1} (pulled into S_t), or S_0 when from_s0
  int with_drag;         // add kappa grad D(S_t)
  int from_s0;
  int t;                 // the collision C(S_t) -> P_t: under the random field when t < field_steps
  const float *maps;     // random body-force fields (nullable)
};

// body force of the collision C(S_t) at node n of a clone: beta (1 + eps map)
// while the run's field acts (t < field_steps), else beta, as the forward
template <typename T>
__device__ __forceinline__ T adj_beta(const RunDev &R, const AdjArgs &a, int clone, int n) {
  if (!(R.field_mode && a.maps && a.t < R.field_steps)) return (T)R.beta;
  const float m = a.maps[R.map_base + (long long)clone * R.nodes + n];
  if (sizeof(T) == 8) return (T)(R.beta * (1.0 + R.field_eps * (double)m));
  return (T)field_beta_f32(R.f_beta, R.f_field_eps, m);
}

__device__ __forceinline__ int adj_locate(const RunDev *runs, int nruns, int &clone, int &n) {
  const int b = blockIdx.x;
  int r = 0;
  while (r + 1 < nruns && b >= runs[r + 1].block_base) r++;
  const RunDev &R = runs[r];
  const int local = b - R.block_base;
  clone = local / R.blocks_per_clone;
  n = (local - clone * R.blocks_per_clone) * blockDim.x + threadIdx.x;
  return r;
}

// gradient of this node's drag contribution w.r.t. its nine populations
// (f or g = f - w, the same derivative), times kappa
template <typename T>
__device__ __forceinline__ void drag_grad(const RunDev &R, int x, int y, const T S[9], T kappa,
                                          T out[9]) {
  if (R.drag_mode == 1) {
    const int m = bounce_mask(R, x, y);
#pragma unroll
    for (int k = 0; k < 9; k++) out[k] = ((m >> k) & 1) ? kappa * T(-2 * cx_of(k)) : T(0);
    return;
  }
  T rho, jx = (S[1] - S[3]) + ((S[5] - S[7]) + (S[8] - S[6]));
  T jy = (S[2] - S[4]) + ((S[5] - S[7]) + (S[6] - S[8]));
  T sum = ((S[0] + (S[1] + S[3])) + (S[2] + S[4])) + ((S[5] + S[7]) + (S[6] + S[8]));
  rho = (sizeof(T) == 8 ? sum : T(1) + sum);
  const T ux = jx / rho, uy = jy / rho;
  const T c = (T)R.cforce;
  T wx = 0, wxy = 0;  // weights of dPi_xx and dPi_xy
  T wr = 0;           // weight of d(rho/3)
  if (x == R.xmin) { wr += T(1); wx += c; }
  if (x == R.xmax) { wr -= T(1); wx -= c; }
  if (y == R.ymax) wxy -= c;
  if (y == R.ymin) wxy += c;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const T cx = (T)cx_of(k), cy = (T)cy_of(k);
    const T dpxx = (cx != T(0) ? T(1) : T(0)) - T(1) / T(3) - (T(2) * ux * cx - ux * ux);
    const T dpxy = cx * cy - cx * uy - cy * ux + ux * uy;
    out[k] = kappa * (wr * (T(1) / T(3)) + wx * dpxx + wxy * dpxy);
  }
}

// sigma_S = J_C(S)^T pi for the BGK + Guo collision of clbm_physics.cuh.
// The collision is (1 - omega) I plus a function of rho, ux, uy, so
// J^T pi = (1 - omega) pi + A + c_k (Bx, By) with G = d/d(rho, ux, uy) of
// sum_k pi_k (omega feq_k + F_k).  Written through the weighted moments of pi
// (P0 = sum w pi, Px = sum w cx pi, ..., Pxy = sum w cx cy pi), the sums over
// k of the per-k derivatives collapse to a few products:
//   G0 = omega (P0 (1 - u2) + 3 (ux Px + uy Py) + 4.5 (ux^2 Pxx + 2 ux uy Pxy + uy^2 Pyy))
//   Gx = omega rho (3 Px + 9 (ux Pxx + uy Pxy) - 3 ux P0) + cf beta (9 Pxx - 3 P0)
//   Gy = omega rho (3 Py + 9 (ux Pxy + uy Pyy) - 3 uy P0) + 9 cf beta Pxy
// (u2 = 1.5 |u|^2, cf the Guo prefactor, feq and F as in collide_ref64).
template <typename T>
__device__ __forceinline__ void collide_adjoint(const RunDev &R, const T S[9], const T pi[9], T beta,
                                                T out[9]) {
  const T omega = (T)R.omega, om1 = T(1) - omega;
  const T cf = (T)R.cforce;
  T sum = ((S[0] + (S[1] + S[3])) + (S[2] + S[4])) + ((S[5] + S[7]) + (S[6] + S[8]));
  const T rho = (sizeof(T) == 8 ? sum : T(1) + sum);
  const T jx = (S[1] - S[3]) + ((S[5] - S[7]) + (S[8] - S[6]));
  const T jy = (S[2] - S[4]) + ((S[5] - S[7]) + (S[6] - S[8]));
  const T ux = (jx + T(0.5) * beta) / rho, uy = jy / rho;
  const T u2 = T(1.5) * (ux * ux + uy * uy);
  const T wa = T(1) / T(9), wd = T(1) / T(36);
  const T a13 = pi[1] + pi[3], a24 = pi[2] + pi[4];
  const T dsum = (pi[5] + pi[7]) + (pi[6] + pi[8]);
  const T P0 = T(4) / T(9) * pi[0] + wa * (a13 + a24) + wd * dsum;
  const T Px = wa * (pi[1] - pi[3]) + wd * ((pi[5] - pi[7]) + (pi[8] - pi[6]));
  const T Py = wa * (pi[2] - pi[4]) + wd * ((pi[5] - pi[7]) + (pi[6] - pi[8]));
  const T Pxx = wa * a13 + wd * dsum;
  const T Pyy = wa * a24 + wd * dsum;
  const T Pxy = wd * ((pi[5] + pi[7]) - (pi[6] + pi[8]));
  const T G0 = omega * (P0 * (T(1) - u2) + T(3) * (ux * Px + uy * Py) +
                        T(4.5) * (ux * ux * Pxx + T(2) * ux * uy * Pxy + uy * uy * Pyy));
  const T Gx = omega * rho * (T(3) * Px + T(9) * (ux * Pxx + uy * Pxy) - T(3) * ux * P0) +
               cf * beta * (T(9) * Pxx - T(3) * P0);
  const T Gy = omega * rho * (T(3) * Py + T(9) * (ux * Pxy + uy * Pyy) - T(3) * uy * P0) + T(9) * cf * beta * Pxy;
  const T inv = T(1) / rho;
  const T A = G0 - (ux * Gx + uy * Gy) * inv;
  const T Bx = Gx * inv, By = Gy * inv;
#pragma unroll
  for (int k = 0; k < 9; k++) out[k] = om1 * pi[k] + A + (T)cx_of(k) * Bx + (T)cy_of(k) * By;
}

template <bool F64>
__global__ void __launch_bounds__(STEP_BLOCK) k_adj_step(AdjArgs a) {
  using T = real_t<F64>;
  int clone, n;
  const int r = adj_locate(a.runs, a.nruns, clone, n);
  const RunDev &R = a.runs[r];
  if (n >= R.nodes || clone >= R.nclones) return;
  const long long plane = R.plane;
  const long long cb = R.pop_base + (long long)clone * 9 * plane;
  const T *sig = (const T *)a.sigma_in + cb;
  const T *P = (const T *)a.P + cb;
  T *out = (T *)a.sigma_out + cb;
  const int W = R.W, y = (int)__umulhi((unsigned)n, R.div_w), x = n - y * W;
  const bool in_box = x >= R.xmin && x <= R.xmax && y >= R.ymin && y <= R.ymax;
  const int mask = (in_box || y == 0 || y == R.H - 1) ? bounce_mask(R, x, y) : 0;
  if (mask & 512) {
#pragma unroll
    for (int k = 0; k < 9; k++) out[k * plane + n] = T(0);
    return;
  }
  const int xl = (x == 0) ? W - 1 : x - 1, xr = (x == W - 1) ? 0 : x + 1;
  const int row = y * W;
  T S[9], pi[9];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const int cx = cx_of(k), cy = cy_of(k);
    // S_t(n,k) = P_{t-1}(n - c_k, k), or P_{t-1}(n, opp k) when bounced
    if (a.from_s0) {
      S[k] = P[k * plane + n];
    } else {
      const int sx = cx == 1 ? xl : (cx == -1 ? xr : x);
      const int srow = cy == 1 ? row - W : (cy == -1 ? row + W : row);
      S[k] = ((mask >> k) & 1) ? P[opp_of(k) * plane + n] : P[k * plane + srow + sx];
    }
    // P(n,k) is read by slot (n, opp k) when that slot bounces, else by (n + c_k, k)
    const int ok = opp_of(k);
    if ((mask >> ok) & 1) {
      pi[k] = sig[ok * plane + n];
    } else {
      const int tx = cx == 1 ? xr : (cx == -1 ? xl : x);
      const int trow = cy == 1 ? row + W : (cy == -1 ? row - W : row);
      pi[k] = sig[k * plane + trow + tx];
    }
  }
  T o[9];
  collide_adjoint<T>(R, S, pi, adj_beta<T>(R, a, clone, n), o);
  if (a.with_drag && in_box) {
    T dg[9];
    drag_grad<T>(R, x, y, S, (T)(R.dt * R.force_scale), dg);
#pragma unroll
    for (int k = 0; k < 9; k++) o[k] += dg[k];
  }
#pragma unroll
  for (int k = 0; k < 9; k++) out[k * plane + n] = o[k];
}

// sigma_T = kappa grad D(Pull(P_{T-1})), zero away from the perimeter
template <bool F64>
__global__ void __launch_bounds__(STEP_BLOCK) k_adj_init(AdjArgs a) {
  using T = real_t<F64>;
  int clone, n;
  const int r = adj_locate(a.runs, a.nruns, clone, n);
  const RunDev &R = a.runs[r];
  if (n >= R.nodes || clone >= R.nclones) return;
  const long long plane = R.plane;
  const long long cb = R.pop_base + (long long)clone * 9 * plane;
  const T *P = (const T *)a.P + cb;
  T *out = (T *)a.sigma_out + cb;
  const int W = R.W, y = (int)__umulhi((unsigned)n, R.div_w), x = n - y * W;
  const bool in_box = x >= R.xmin && x <= R.xmax && y >= R.ymin && y <= R.ymax;
  const int mask = in_box ? bounce_mask(R, x, y) : 0;
  if (!in_box || (mask & 512)) {
#pragma unroll
    for (int k = 0; k < 9; k++) out[k * plane + n] = T(0);
    return;
  }
  const int xl = (x == 0) ? W - 1 : x - 1, xr = (x == W - 1) ? 0 : x + 1;
  const int row = y * W;
  T S[9];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const int cx = cx_of(k), cy = cy_of(k);
    const int sx = cx == 1 ? xl : (cx == -1 ? xr : x);
    const int srow = cy == 1 ? row - W : (cy == -1 ? row + W : row);
    S[k] = ((mask >> k) & 1) ? P[opp_of(k) * plane + n] : P[k * plane + srow + sx];
  }
  T dg[9];
  drag_grad<T>(R, x, y, S, (T)(R.dt * R.force_scale), dg);
#pragma unroll
  for (int k = 0; k < 9; k++) out[k * plane + n] = dg[k];
}

cudaError_t launch_adj_init(bool f64, const RunDev *runs, int nruns, const void *P, void *sigma,
                            int blocks, cudaStream_t s) {
  AdjArgs a{runs, nruns, nullptr, sigma, P, 1, 0, 0, nullptr};
  if (f64)
    k_adj_init<true><<<blocks, STEP_BLOCK, 0, s>>>(a);
  else
    k_adj_init<false><<<blocks, STEP_BLOCK, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_adj_step(bool f64, const RunDev *runs, int nruns, const void *sigma_in,
                            void *sigma_out, const void *P, bool with_drag, bool from_s0, int t,
                            const float *maps, int blocks, cudaStream_t s) {
  AdjArgs a{runs, nruns, sigma_in, sigma_out, P, with_drag ? 1 : 0, from_s0 ? 1 : 0, t, maps};
  if (f64)
    k_adj_step<true><<<blocks, STEP_BLOCK, 0, s>>>(a);
  else
    k_adj_step<false><<<blocks, STEP_BLOCK, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace clbm
