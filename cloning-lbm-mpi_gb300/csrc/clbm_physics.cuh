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
//   g*_k  = (1 - omega) g_k + omega geq_k + F_k

// FP32 body force of a node under a random field: beta (1 + eps m), with
// explicit rounding steps so that no kernel contracts or reorders it
// differently (the streaming and cluster-resident kernels must agree bit for
// bit); eps = 0 gives beta exactly.
__device__ __forceinline__ float field_beta_f32(float beta, float eps, float m) {
  return __fmul_rn(beta, __fmaf_rn(eps, m, 1.0f));
}

namespace f32op {
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
}  // namespace f32op

// Packed FP32 arithmetic (Blackwell f32x2): each lane is the IEEE
// round-to-nearest operation of its scalar counterpart, so a packed
// expression gives the same bits as the two scalar ones it replaces.
namespace f32x2op {
__device__ __forceinline__ float lo(f2_t v) { return __uint_as_float((unsigned)v); }
__device__ __forceinline__ float hi(f2_t v) { return __uint_as_float((unsigned)(v >> 32)); }
__device__ __forceinline__ f2_t add(f2_t a, f2_t b) {
  f2_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2_t sub(f2_t a, f2_t b) {
  f2_t d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2_t mul(f2_t a, f2_t b) {
  f2_t d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2_t fma(f2_t a, f2_t b, f2_t c) {
  f2_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
}  // namespace f32x2op

// 1/x by the hardware reciprocal approximation (the value x / y takes in
// fast approximate division for x = 1, without its range fix-ups: x here is
// a density near 1)
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// The collision organised by opposite pairs (k, opp k): they share |c.u|, so
// with e = c_k.u the equilibria split into an even part
// w (drho + rho (4.5 e^2 - 1.5 u^2)) and an odd part +-3 w rho e, and the
// Guo terms into w fb (9 cx e - 3 ux) and +-3 w fb cx.  Returns drho.
//
// Free of systematic rounding bias in the momentum.  The equilibrium
// momentum rho u (~0.05) is ~10^4 times the body force added per step
// (~1e-6), so a rounding that errs the same way at every node and step,
// even by a fraction of an ulp, acts as a spurious body force of a sizeable
// fraction of the real one and the flow drifts over an interval series.
// Three such roundings are avoided:
//  * the velocity shift: jx + beta/2 rounds a fixed offset onto the grid of
//    jx, the same error at every node; ux = jx/rho + (beta/2)/rho is formed
//    by one fused multiply-add of the exact product jx * (1/rho) instead;
//  * the weights: the odd parts carry the momentum through the coefficients
//    3 w omega, and float(1/9) is 7.5e-9 too large, which puts 7.5e-9 rho u
//    of momentum into every node and step; the coefficients here are
//    c13 ~ omega/3 and c2 ~ omega/12 with omega' = 2 c13 + 4 c2 and
//    om1 = 1 - omega' exact, so the odd parts relax the momentum by exactly
//    the factor the (1 - omega') g_k terms leave;
//  * rho near 1: omega * (3 rho) rounds a near-constant product the same way
//    at many nodes; the odd parts use rho u = ux + drho ux instead, a fused
//    multiply-add of an exact product.
// The remaining roundings act on operands with effectively random low bits.
// Every operation is an explicitly rounded intrinsic (the fused
// multiply-adds chosen here, none left to the compiler), so the result is the
// same bit for bit in every kernel that inlines it.
//
// The four direction pairs are evaluated two at a time in packed f32x2
// arithmetic: the axis pairs (1,3) and (2,4) in lanes 0 and 1 with e = (ux,
// uy), the diagonal pairs (5,7) and (6,8) with e = (ux + uy, uy - ux).  Lane
// 1 of the axis Guo term is fma(0, uy, fx) = fx and its odd part
// fma(c13, ty, -0) = c13 ty, so every lane is the scalar expression of its
// pair; the k -> (k, opp k) sums and differences of the moments are packed
// the same way.  k holds the run's constants in lane pairs (F32Pairs).
__device__ __forceinline__ float collide_f32_pairs(const float g[9], float out[9], float omega,
                                                   const F32Force &f, const F32Pairs &k) {
  using namespace f32op;
  namespace X = f32x2op;
  const f2_t g12 = f2_bits(g[1], g[2]), g34 = f2_bits(g[3], g[4]);
  const f2_t g56 = f2_bits(g[5], g[6]), g78 = f2_bits(g[7], g[8]);
  const f2_t a1324 = X::add(g12, g34), d1324 = X::sub(g12, g34);  // (g1 +- g3, g2 +- g4)
  const f2_t a5768 = X::add(g56, g78);                            // (g5 + g7, g6 + g8)
  const float s57 = sub(g[5], g[7]), t86 = sub(g[8], g[6]);
  const float drho = add(add(add(g[0], X::lo(a1324)), X::hi(a1324)), add(X::lo(a5768), X::hi(a5768)));
  // jy's s57 + (g6 - g8) is s57 - t86: the rounded g6 - g8 is exactly -t86
  const float jx = add(X::lo(d1324), add(s57, t86));
  const float jy = add(X::hi(d1324), sub(s57, t86));
  const float rho = add(1.0f, drho);
  // 1/(1 + drho): the hardware approximation r0 of 1/rho refined by one
  // Newton-Raphson step on the unrounded density, r0 + r0 ((1 - r0) - drho r0)
  // (1 - r0 is exact: r0 is near 1)
  const float r0 = rcp_approx(rho);
  const float inv = fma(r0, fma(-drho, r0, sub(1.0f, r0)), r0);
  const float ux = fma(jx, inv, mul(f.hb, inv));
  const float uy = mul(jy, inv);
  const float tx = fma(drho, ux, ux), ty = fma(drho, uy, uy);  // rho u
  const float u2 = mul(1.5f, fma(ux, ux, mul(uy, uy)));
  const float base = fma(-rho, u2, drho);  // even part before the e^2 term (per unit weight)
  const float fx = mul(f.fbm3, ux);         // Guo even part for cx = 0 (per unit weight)
  // k = 0
  out[0] = fma(X::lo(k.om1), g[0], mul(4.0f / 9.0f, fma(omega, base, fx)));
  const float r45 = mul(4.5f, rho);
  const f2_t R45 = f2_bits(r45, r45), BASE = f2_bits(base, base), FX = f2_bits(fx, fx);
  // axis pairs: lane 0 (1,3) e = ux, cx = 1; lane 1 (2,4) e = uy, cx = 0
  {
    const f2_t e = f2_bits(ux, uy), t = f2_bits(tx, ty);
    const f2_t ev = X::mul(k.w9, X::fma(k.omega, X::fma(X::mul(R45, e), e, BASE), X::fma(k.fb9_0, e, FX)));
    const f2_t od = X::fma(k.c13, t, k.f13_0);
    const f2_t o12 = X::fma(k.om1, g12, X::add(ev, od)), o34 = X::fma(k.om1, g34, X::sub(ev, od));
    out[1] = X::lo(o12);
    out[2] = X::hi(o12);
    out[3] = X::lo(o34);
    out[4] = X::hi(o34);
  }
  // diagonal pairs: lane 0 (5,7) e = ux + uy, cx = 1; lane 1 (6,8) e = uy - ux, cx = -1
  {
    const f2_t e = f2_bits(add(ux, uy), sub(uy, ux)), t = f2_bits(add(tx, ty), sub(ty, tx));
    const f2_t ev = X::mul(k.w36, X::fma(k.omega, X::fma(X::mul(R45, e), e, BASE), X::fma(k.fb9_m, e, FX)));
    const f2_t od = X::fma(k.c2, t, k.f2_m);
    const f2_t o56 = X::fma(k.om1, g56, X::add(ev, od)), o78 = X::fma(k.om1, g78, X::sub(ev, od));
    out[5] = X::lo(o56);
    out[6] = X::hi(o56);
    out[7] = X::lo(o78);
    out[8] = X::hi(o78);
  }
  return drho;
}

// The FP32 collision of one node of run R; field: the node's random-field
// value, or nullptr under the uniform body force.
__device__ __forceinline__ float collide_f32_run(const RunDev &R, const float S[9], float P[9],
                                                 const float *field = nullptr, float feps = 0.f) {
  if (field) {
    const F32Force f = f32_force(field_beta_f32(R.f_beta, feps, *field), R.f_cforce);
    F32Pairs k = R.f_pairs;
    f32_pairs_force(k, f);
    return collide_f32_pairs(S, P, R.f_omega, f, k);
  }
  return collide_f32_pairs(S, P, R.f_omega, R.f_force, R.f_pairs);
}

// Drag terms from shifted populations, rest parts removed analytically:
//   pi_xx = sum_{cx!=0} g - drho/3 - rho ux^2,  pi_xy = g5 - g6 + g7 - g8 - rho ux uy
// and the West/East rho/3 becomes drho/3 (the +-1/3 cancel between sides).
// (explicitly rounded like collide_f32_pairs)
__device__ __forceinline__ void pi_f32(const float g[9], float &drho_o, float &pxx, float &pxy) {
  using namespace f32op;
  const float a57 = add(g[5], g[7]), a68 = add(g[6], g[8]);
  const float s57 = sub(g[5], g[7]);
  const float drho = add(add(add(g[0], add(g[1], g[3])), add(g[2], g[4])), add(a57, a68));
  const float jx = add(sub(g[1], g[3]), add(s57, sub(g[8], g[6])));
  const float jy = add(sub(g[2], g[4]), add(s57, sub(g[6], g[8])));
  const float rho = add(1.0f, drho);
  const float ux = __fdiv_rn(jx, rho), uy = __fdiv_rn(jy, rho);
  const float sxx = add(add(g[1], g[3]), add(a57, a68));
  const float rux = mul(rho, ux);
  drho_o = drho;
  pxx = fma(-rux, ux, fma(-drho, 1.0f / 3.0f, sxx));
  pxy = fma(-rux, uy, sub(a57, a68));
}

// Momentum-exchange drag of one perimeter node.  A slot k that the square
// bounces back holds S(n,k) = P(n, opp k): the population that left n towards
// the solid along c_{opp k} and came back along c_k, handing the body
// c_{opp k} P - c_k S = -2 c_k S of momentum.  The x parts are summed in k
// order (c_kx = 0 slots carry none).  FP64 on f; FP32 on the shifted g, whose
// missing rest parts -2 c_kx w_k cancel over the perimeter (West against East
// row by row, corner against corner, +-c_x pairs on North and South).
template <bool F64>
__device__ __forceinline__ typename std::conditional<F64, double, float>::type me_node_term(
    const typename std::conditional<F64, double, float>::type S[9], int mask) {
  typename std::conditional<F64, double, float>::type v = 0;
#pragma unroll
  for (int k = 1; k < 9; k++) {
    if (cx_of(k) == 0 || !((mask >> k) & 1)) continue;
    if constexpr (F64) {
      const double s2 = DADD(S[k], S[k]);
      v = cx_of(k) < 0 ? DADD(v, s2) : DSUB(v, s2);
    } else {
      const float s2 = __fadd_rn(S[k], S[k]);
      v = cx_of(k) < 0 ? __fadd_rn(v, s2) : __fsub_rn(v, s2);
    }
  }
  return v;
}

// Drag terms of one perimeter node, stored at [term][clone] so that the
// reduction reads them coalesced: West (x = xmin, index y - ymin), East,
// North (y = ymax, index x - xmin), South.  Stress integration (drag_mode 0):
// FP64 the reference's per-node expressions (force.cpp:48, :78, :108, :138),
// FP32 a shifted variant without the +-1/3 that cancel between West and East.
// Momentum exchange (drag_mode 1): the node's me_node_term in its West or
// East slot (corners included) or its North or South slot, 0 in the North and
// South slots of the corners, so every node counts once.
template <bool F64>
__device__ __forceinline__ void store_drag_terms(
    const RunDev &R, const typename std::conditional<F64, double, float>::type S[9], int x, int y,
    int clone, typename std::conditional<F64, double, float>::type *T) {
  const int sy = R.ymax - R.ymin, sx = R.xmax - R.xmin;
  const int nc = R.nclones;
  if (R.drag_mode == 1) {
    const auto v = me_node_term<F64>(S, bounce_mask(R, x, y));
    const bool corner_x = x == R.xmin || x == R.xmax;
    if (x == R.xmin) T[(long long)(y - R.ymin) * nc + clone] = v;
    if (x == R.xmax) T[(long long)(sy + 1 + y - R.ymin) * nc + clone] = v;
    if (y == R.ymax) T[(long long)(2 * (sy + 1) + x - R.xmin) * nc + clone] = corner_x ? 0 : v;
    if (y == R.ymin) T[(long long)(2 * (sy + 1) + sx + 1 + x - R.xmin) * nc + clone] = corner_x ? 0 : v;
    return;
  }
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
    west = __fmaf_rn(drho, 1.0f / 3.0f, __fmul_rn(c, pxx));
    east = -west;
    north = __fmul_rn(-c, pxy);
    south = __fmul_rn(c, pxy);
  }
  if (x == R.xmin) T[(long long)(y - R.ymin) * nc + clone] = west;
  if (x == R.xmax) T[(long long)(sy + 1 + y - R.ymin) * nc + clone] = east;
  if (y == R.ymax) T[(long long)(2 * (sy + 1) + x - R.xmin) * nc + clone] = north;
  if (y == R.ymin) T[(long long)(2 * (sy + 1) + sx + 1 + x - R.xmin) * nc + clone] = south;
}

}  // namespace clbm
