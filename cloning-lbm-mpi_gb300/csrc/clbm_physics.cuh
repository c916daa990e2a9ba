// clbm_physics.cuh -- per-node D2Q9 BGK physics used by every kernel.
//
// Two arithmetic policies:
//  * ref64: FP64 in the reference's exact operation order with explicit
//    round-to-nearest intrinsics, so nothing is contracted into an FMA; the
//    results are bit-identical to the reference's g++ build
//    (src/lbm_src/streamCollCompute.cpp:19-41, src/lbm_src/force.cpp:26-48).
//    Terms that the reference multiplies by a lattice velocity of 0 are
//    dropped and the +-1 products are written as additions/subtractions: both
//    are exact, and only the sign of an exactly-zero intermediate could differ.
//  * f32: FP32 populations stored as g = f - w[k] ("shifted"), collision and
//    drag terms evaluated on the shifted values so that the O(1) rest parts
//    cancel analytically instead of in rounding.
#pragma once
#include <type_traits>

#include "clbm_common.cuh"

namespace clbm {

// ---------------------------------------------------------------- ref64 ----
#define DADD __dadd_rn
#define DSUB __dsub_rn
#define DMUL __dmul_rn
#define DDIV __ddiv_rn

struct Moments64 {
  double rho, jx, jy;
};

// rho, jx, jy summed in the reference's k order (streamCollCompute.cpp:21-27)
__device__ __forceinline__ Moments64 moments_ref64(const double f[9]) {
  Moments64 m;
  double r = f[0];
#pragma unroll
  for (int k = 1; k < 9; k++) r = DADD(r, f[k]);
  m.rho = r;
  m.jx = DADD(DSUB(DSUB(DADD(DSUB(f[1], f[3]), f[5]), f[6]), f[7]), f[8]);
  m.jy = DSUB(DSUB(DADD(DADD(DSUB(f[2], f[4]), f[5]), f[6]), f[7]), f[8]);
  return m;
}

// c_k . u for the nine directions, as the reference evaluates cx*ux + cy*uy
__device__ __forceinline__ double eu_ref64(int k, double ux, double uy) {
  switch (k) {
    case 0: return 0.0;
    case 1: return ux;
    case 2: return uy;
    case 3: return -ux;
    case 4: return -uy;
    case 5: return DADD(ux, uy);
    case 6: return DADD(-ux, uy);
    case 7: return DADD(-ux, -uy);
    default: return DADD(ux, -uy);
  }
}

// w[k]*rho*(1 + 3 eu + 4.5 eu^2 + u2), u2 = -1.5 |u|^2 (streamCollCompute.cpp:32-34)
__device__ __forceinline__ double feq_ref64(int k, double rho, double eu, double u2) {
  const double eueu = DMUL(DMUL(4.5, eu), eu);
  return DMUL(DMUL(w_of(k), rho), DADD(DADD(DADD(1.0, DMUL(3.0, eu)), eueu), u2));
}

// BGK collision with the Guo forcing term, velocity shifted by beta/(2 rho)
// (streamCollCompute.cpp:28-37).  wcb[k] = (w[k]*(1 - omega/2))*beta.
__device__ __forceinline__ void collide_ref64(const double f[9], double out[9], double beta,
                                              const double wcb[9], double omega,
                                              double om1, double *rho_o = nullptr,
                                              double *ux_o = nullptr, double *uy_o = nullptr) {
  const Moments64 m = moments_ref64(f);
  const double ux = DADD(DDIV(m.jx, m.rho), DDIV(DMUL(0.5, beta), m.rho));
  const double uy = DDIV(m.jy, m.rho);
  const double u2 = DMUL(-1.5, DADD(DMUL(ux, ux), DMUL(uy, uy)));
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const double eu = eu_ref64(k, ux, uy);
    const double feq = feq_ref64(k, m.rho, eu, u2);
    const int c = cx_of(k);
    // 3*(cx - ux) + 9*cx*eu
    double drive;
    if (c == 0)
      drive = DMUL(3.0, -ux);
    else if (c == 1)
      drive = DADD(DMUL(3.0, DSUB(1.0, ux)), DMUL(9.0, eu));
    else
      drive = DADD(DMUL(3.0, DSUB(-1.0, ux)), DMUL(-9.0, eu));
    drive = DMUL(wcb[k], drive);
    out[k] = DADD(DADD(DMUL(f[k], om1), DMUL(feq, omega)), drive);
  }
  if (rho_o) {
    *rho_o = m.rho;
    *ux_o = ux;
    *uy_o = uy;
  }
}

// Non-equilibrium second moments with the UNshifted velocity
// (force.cpp:26-46): pi_xx = sum fneq cx cx, pi_xy = sum fneq cx cy.
__device__ __forceinline__ void pi_ref64(const double f[9], double &rho, double &pxx,
                                         double &pxy) {
  const Moments64 m = moments_ref64(f);
  const double uy = DDIV(m.jy, m.rho);
  const double ux = DDIV(m.jx, m.rho);
  const double u2 = DMUL(-1.5, DADD(DMUL(ux, ux), DMUL(uy, uy)));
  double fneq[9];
#pragma unroll
  for (int k = 1; k < 9; k++) fneq[k] = DSUB(f[k], feq_ref64(k, m.rho, eu_ref64(k, ux, uy), u2));
  rho = m.rho;
  pxx = DADD(DADD(DADD(DADD(DADD(fneq[1], fneq[3]), fneq[5]), fneq[6]), fneq[7]), fneq[8]);
  pxy = DSUB(DADD(DSUB(fneq[5], fneq[6]), fneq[7]), fneq[8]);
}

// ------------------------------------------------------------------ f32 ----
// Shifted populations g = f - w.  With drho = rho - 1:
//   geq_k = feq_k - w_k = w_k (drho + rho (3 eu + 4.5 eu^2 - 1.5 u^2))
//   g*_k  = g_k + omega (geq_k - g_k) + F_k
__device__ __forceinline__ void collide_f32(const float g[9], float out[9], float beta,
                                            float omega, float cforce, float *rho_o = nullptr,
                                            float *ux_o = nullptr, float *uy_o = nullptr) {
  const float drho = ((g[0] + (g[1] + g[3])) + (g[2] + g[4])) + ((g[5] + g[7]) + (g[6] + g[8]));
  const float jx = (g[1] - g[3]) + ((g[5] - g[7]) + (g[8] - g[6]));
  const float jy = (g[2] - g[4]) + ((g[5] - g[7]) + (g[6] - g[8]));
  const float rho = 1.0f + drho;
  const float inv = 1.0f / rho;
  const float ux = (jx + 0.5f * beta) * inv;
  const float uy = jy * inv;
  const float u2 = 1.5f * (ux * ux + uy * uy);
  const float fb = cforce * beta;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const int cx = cx_of(k), cy = cy_of(k);
    const float eu = (float)cx * ux + (float)cy * uy;
    const float wk = (float)w_of(k);
    const float geq = wk * (drho + rho * (eu * (3.0f + 4.5f * eu) - u2));
    const float drive = wk * fb * (3.0f * ((float)cx - ux) + 9.0f * (float)cx * eu);
    out[k] = g[k] + omega * (geq - g[k]) + drive;
  }
  if (rho_o) {
    *rho_o = rho;
    *ux_o = ux;
    *uy_o = uy;
  }
}

// The same collision organised by opposite pairs (k, opp k): they share
// |c.u|, so with e = c_k.u the equilibria split into an even part
// w (drho + rho (4.5 e^2 - 1.5 u^2)) and an odd part +-3 w rho e, and the
// Guo terms into w fb (9 cx e - 3 ux) and +-3 w fb cx.  Returns drho.
__device__ __forceinline__ float collide_f32_pairs(const float g[9], float out[9], float beta,
                                                   float omega, float cforce) {
  const float drho = ((g[0] + (g[1] + g[3])) + (g[2] + g[4])) + ((g[5] + g[7]) + (g[6] + g[8]));
  const float jx = (g[1] - g[3]) + ((g[5] - g[7]) + (g[8] - g[6]));
  const float jy = (g[2] - g[4]) + ((g[5] - g[7]) + (g[6] - g[8]));
  const float rho = 1.0f + drho;
  const float inv = __frcp_rn(rho);
  const float ux = (jx + 0.5f * beta) * inv;
  const float uy = jy * inv;
  const float u2 = 1.5f * (ux * ux + uy * uy);
  const float fb = cforce * beta;
  const float om1 = 1.0f - omega;
  const float base = drho - rho * u2;      // even part before the e^2 term (per unit weight)
  const float fx = -3.0f * fb * ux;        // Guo even part for cx = 0 (per unit weight)
  // k = 0
  out[0] = om1 * g[0] + (4.0f / 9.0f) * (omega * base + fx);
  const float r45 = 4.5f * rho, r3 = 3.0f * rho;
  // axis pairs (1,3): e = ux, cx = 1; (2,4): e = uy, cx = 0
  {
    const float w = 1.0f / 9.0f;
    const float e = ux;
    const float ev = w * (omega * (base + r45 * e * e) + (9.0f * fb * e + fx));
    const float od = w * (omega * r3 * e + 3.0f * fb);
    out[1] = om1 * g[1] + (ev + od);
    out[3] = om1 * g[3] + (ev - od);
  }
  {
    const float w = 1.0f / 9.0f;
    const float e = uy;
    const float ev = w * (omega * (base + r45 * e * e) + fx);
    const float od = w * (omega * r3 * e);
    out[2] = om1 * g[2] + (ev + od);
    out[4] = om1 * g[4] + (ev - od);
  }
  // diagonal pairs (5,7): e = ux + uy, cx = 1; (6,8): e = uy - ux, cx = -1
  {
    const float w = 1.0f / 36.0f;
    const float e = ux + uy;
    const float ev = w * (omega * (base + r45 * e * e) + (9.0f * fb * e + fx));
    const float od = w * (omega * r3 * e + 3.0f * fb);
    out[5] = om1 * g[5] + (ev + od);
    out[7] = om1 * g[7] + (ev - od);
  }
  {
    const float w = 1.0f / 36.0f;
    const float e = uy - ux;
    const float ev = w * (omega * (base + r45 * e * e) + (-9.0f * fb * e + fx));
    const float od = w * (omega * r3 * e - 3.0f * fb);
    out[6] = om1 * g[6] + (ev + od);
    out[8] = om1 * g[8] + (ev - od);
  }
  return drho;
}

// Drag terms from shifted populations, rest parts removed analytically:
//   pi_xx = sum_{cx!=0} g - drho/3 - rho ux^2,  pi_xy = g5 - g6 + g7 - g8 - rho ux uy
// and the West/East rho/3 becomes drho/3 (the +-1/3 cancel between sides).
__device__ __forceinline__ void pi_f32(const float g[9], float &drho_o, float &pxx, float &pxy) {
  const float drho = ((g[0] + (g[1] + g[3])) + (g[2] + g[4])) + ((g[5] + g[7]) + (g[6] + g[8]));
  const float jx = (g[1] - g[3]) + ((g[5] - g[7]) + (g[8] - g[6]));
  const float jy = (g[2] - g[4]) + ((g[5] - g[7]) + (g[6] - g[8]));
  const float rho = 1.0f + drho;
  const float ux = jx / rho, uy = jy / rho;
  const float sxx = (g[1] + g[3]) + ((g[5] + g[7]) + (g[6] + g[8]));
  drho_o = drho;
  pxx = sxx - drho * (1.0f / 3.0f) - rho * ux * ux;
  pxy = ((g[5] + g[7]) - (g[6] + g[8])) - rho * ux * uy;
}

// Drag terms of one perimeter node, stored at [term][clone] so that the
// reduction reads them coalesced: West (x = xmin, index y - ymin), East,
// North (y = ymax, index x - xmin), South.  FP64: the reference's per-node
// expressions (force.cpp:48, :78, :108, :138).  FP32: shifted variant without
// the +-1/3 that cancel between West and East.
template <bool F64>
__device__ __forceinline__ void store_drag_terms(
    const RunDev &R, const typename std::conditional<F64, double, float>::type S[9], int x, int y,
    int clone, typename std::conditional<F64, double, float>::type *T) {
  const int sy = R.ymax - R.ymin, sx = R.xmax - R.xmin;
  const int nc = R.nclones;
  typename std::conditional<F64, double, float>::type west, east, north, south;
  if constexpr (F64) {
    double rho, pxx, pxy;
    pi_ref64(S, rho, pxx, pxy);
    const double third = 1. / 3.;
    const double c = R.cforce;
    west = DADD(DMUL(rho, third), DMUL(c, pxx));
    east = DSUB(DMUL(-rho, third), DMUL(c, pxx));
    north = DMUL(-c, pxy);
    south = DMUL(c, pxy);
  } else {
    float drho, pxx, pxy;
    pi_f32(S, drho, pxx, pxy);
    const float c = R.f_cforce;
    west = drho * (1.0f / 3.0f) + c * pxx;
    east = -west;
    north = -c * pxy;
    south = c * pxy;
  }
  if (x == R.xmin) T[(long long)(y - R.ymin) * nc + clone] = west;
  if (x == R.xmax) T[(long long)(sy + 1 + y - R.ymin) * nc + clone] = east;
  if (y == R.ymax) T[(long long)(2 * (sy + 1) + x - R.xmin) * nc + clone] = north;
  if (y == R.ymin) T[(long long)(2 * (sy + 1) + sx + 1 + x - R.xmin) * nc + clone] = south;
}

}  // namespace clbm
