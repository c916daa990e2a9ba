// clbm_common.cuh -- device-side definitions shared by every clbm kernel:
// the D2Q9 lattice, the per-run descriptor table, node geometry (bounce-back
// classification) and the counter-based / emulated random streams.
#pragma once
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

namespace clbm {

// D2Q9 velocities, weights and opposite directions, in the reference's
// numbering (src/mpi_LBM_GK_pops_perturb.cpp:31-32, src/lbm_src/square.cpp:8).
__host__ __device__ constexpr int cx_of(int k) {
  return (k == 1 || k == 5 || k == 8) ? 1 : (k == 3 || k == 6 || k == 7) ? -1 : 0;
}
__host__ __device__ constexpr int cy_of(int k) {
  return (k == 2 || k == 5 || k == 6) ? 1 : (k == 4 || k == 7 || k == 8) ? -1 : 0;
}
__host__ __device__ constexpr int opp_of(int k) {
  return k == 0 ? 0 : (k <= 4 ? ((k + 1) % 4) + 1 : ((k - 3) % 4) + 5);
}
__host__ __device__ constexpr double w_of(int k) {
  return k == 0 ? 4.0 / 9.0 : (k <= 4 ? 1.0 / 9.0 : 1.0 / 36.0);
}
static_assert(opp_of(1) == 3 && opp_of(2) == 4 && opp_of(3) == 1 && opp_of(4) == 2, "opp");
static_assert(opp_of(5) == 7 && opp_of(6) == 8 && opp_of(7) == 5 && opp_of(8) == 6, "opp");

// Device error word bits (written with atomicOr, read by the host).
enum : unsigned {
  ERR_NONFINITE_DRAG = 1u << 0,
  ERR_WEIGHT_OVERFLOW = 1u << 1,
  ERR_BAD_DENSITY = 1u << 2,
  ERR_BAD_PARENT = 1u << 3,
  ERR_RESAMPLE = 1u << 4,
  ERR_TIMEOUT = 1u << 5,
};

// Body-force terms of the FP32 collision for one value of beta:
// hb = beta/2 (velocity shift), fb = cforce beta, fbm3 = -3 fb, fb9 = 9 fb,
// f13 = fb/3 and f2 = fb/12 (the odd Guo terms of the axis and diagonal
// pairs).  Plain IEEE single-precision products, so the host (uniform runs)
// and the device (a random field, per node) get the same bits for one beta.
struct F32Force {
  float hb, fb, fbm3, fb9, f13, f2;
};
__host__ __device__ inline F32Force f32_force(float beta, float cforce) {
#ifdef __CUDA_ARCH__
#define CLBM_FMUL __fmul_rn
#else
#define CLBM_FMUL(a, b) ((float)(a) * (float)(b))
#endif
  F32Force f;
  f.hb = CLBM_FMUL(0.5f, beta);
  f.fb = CLBM_FMUL(cforce, beta);
  f.fbm3 = CLBM_FMUL(-3.0f, f.fb);
  f.fb9 = CLBM_FMUL(9.0f, f.fb);
  f.f13 = CLBM_FMUL(f.fb, 1.0f / 3.0f);
  f.f2 = CLBM_FMUL(f.fb, 1.0f / 12.0f);
#undef CLBM_FMUL
  return f;
}

// Two FP32 values in one 64-bit word, the operand of the packed (f32x2)
// arithmetic: lane 0 in the low half, lane 1 in the high half.
typedef unsigned long long f2_t;
__host__ __device__ inline f2_t f2_bits(float lo, float hi) {
  unsigned l, h;
  memcpy(&l, &lo, 4);
  memcpy(&h, &hi, 4);
  return ((f2_t)h << 32) | l;
}

// Constant operands of the packed FP32 collision (collide_f32_pairs): lane 0
// serves the pairs (1,3) / (5,7), lane 1 the pairs (2,4) / (6,8).
struct F32Pairs {
  f2_t om1, omega, w9, w36, c13, c2;  // (v, v)
  f2_t fb9_0, fb9_m, f13_0, f2_m;     // (fb9, 0), (fb9, -fb9), (f13, -0), (f2, -f2)
};
__host__ __device__ inline void f32_pairs_force(F32Pairs &p, const F32Force &f) {
  p.fb9_0 = f2_bits(f.fb9, 0.0f);
  p.fb9_m = f2_bits(f.fb9, -f.fb9);
  p.f13_0 = f2_bits(f.f13, -0.0f);
  p.f2_m = f2_bits(f.f2, -f.f2);
}
__host__ __device__ inline F32Pairs f32_pairs(float omega, float om1, float c13, float c2, const F32Force &f) {
  F32Pairs p;
  p.om1 = f2_bits(om1, om1);
  p.omega = f2_bits(omega, omega);
  p.w9 = f2_bits(1.0f / 9.0f, 1.0f / 9.0f);
  p.w36 = f2_bits(1.0f / 36.0f, 1.0f / 36.0f);
  p.c13 = f2_bits(c13, c13);
  p.c2 = f2_bits(c2, c2);
  f32_pairs_force(p, f);
  return p;
}

// One independent run (lattice, square, physics, clone block) of a batch.
struct RunDev {
  int W, H;                    // Dx, Dy
  int xmin, xmax, ymin, ymax;  // square, perimeter inclusive
  int nclones;
  int clone_base;              // first global clone index of this run
  int block_base;              // first block of this run in a step grid
  int blocks_per_clone;
  int nterms;                  // drag terms per clone per step
  int nodes;                   // W*H
  unsigned div_w;              // ceil(2^32 / W): y = umulhi(n, div_w)
  int drag_mode;               // 0 stress integration, 1 momentum exchange
  // tile tables of the FP32 step for tiles of 128 / 256 / 512 nodes: first
  // block of this run, tiles per clone and ceil(2^32 / tiles)
  int tile_base[3];
  int tiles[3];
  unsigned tiles_div[3];
  long long pop_base;          // element offset of this run's clone 0
  long long plane;             // elements per population plane (padded)
  long long term_base;         // offset of this run in a step's term slab
  long long snap_base;         // element offset of this run's snapshots
  // physics, FP64 (reference order) and FP32 copies
  double tau, omega, om1, cforce, beta;
  double wcb[9];               // (w[k]*cforce)*beta, the reference's order
  double alpha, force_scale, force_shift, dt, eps;
  // FP32 collision: omega' = 2 c13 + 4 c2 exactly (c13 ~ omega/3 on a 2^-24
  // grid, c2 ~ omega/12 on a 2^-25 grid), om1 = 1 - omega' and
  // cforce = 1 - omega'/2 exactly; f_force = f32_force(f_beta, f_cforce)
  float f_omega, f_om1, f_c13, f_c2, f_cforce, f_beta;
  F32Force f_force;
  F32Pairs f_pairs;            // the same constants packed for the f32x2 collision
  int perturb_mode, resample_mode, ranks, nsnap;
  unsigned long long seed;
  unsigned run_id;
  int pad2_;
  // Gaussian random body-force field (forcing variant)
  int field_mode, field_steps;
  int M1, M2;                  // embedding sizes 2W-1, 2H-1
  double field_eps;
  float f_field_eps, f_pad2;
  long long map_base;          // element offset of clone 0's map (W*H floats per clone)
  long long spec_base;         // offset of the sqrt-spectrum (M1*M2 floats)
  long long tw1_base, tw2_base;// offsets of the twiddle tables (complex floats)
  long long y_base;            // offset of the stage-1 buffer (W*M2 complex per clone)
  long long fa_base;           // float offset of the stage-1 DFT operand image (tensor cores)
  int f_mpad, f_kchunks;       // its rows (2W rounded up to 128) and 32-wide K chunks
  int fna, fnb;                // modes kept: rows a of the embedding, columns b
  long long flist_base;        // offset of their index lists (a list, then b list)
};

// Bounce-back classification of node (x,y): bit k set means the outgoing
// slot k of this node is written by half-way bounce-back (channel walls,
// src/lbm_src/domain_noSlipWalls.cpp:6-22; square perimeter,
// src/lbm_src/square.cpp:24-50), bit 9 means the node is inside the square
// and is reset to w[k] (pops driver :430-439).
__host__ __device__ inline int bounce_mask(const RunDev &r, int x, int y) {
  int m = 0;
  if (y == r.H - 1) m |= (1 << 4) | (1 << 7) | (1 << 8);
  if (y == 0) m |= (1 << 2) | (1 << 5) | (1 << 6);
  const bool inx = x > r.xmin && x < r.xmax;
  const bool iny = y > r.ymin && y < r.ymax;
  if (inx && y == r.ymin) m |= (1 << 7) | (1 << 4) | (1 << 8);
  if (inx && y == r.ymax) m |= (1 << 5) | (1 << 2) | (1 << 6);
  if (iny && x == r.xmin) m |= (1 << 6) | (1 << 3) | (1 << 7);
  if (iny && x == r.xmax) m |= (1 << 8) | (1 << 1) | (1 << 5);
  if (x == r.xmin && y == r.ymin) m |= 1 << 7;
  if (x == r.xmin && y == r.ymax) m |= 1 << 6;
  if (x == r.xmax && y == r.ymax) m |= 1 << 5;
  if (x == r.xmax && y == r.ymin) m |= 1 << 8;
  if (inx && iny) m |= 1 << 9;
  return m;
}

// ---- Philox4x32-10 (Salmon et al., SC'11) -------------------------------
__host__ __device__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int round = 0; round < 10; round++) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
    const uint32_t n1 = (uint32_t)p1;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    const uint32_t n3 = (uint32_t)p0;
    c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// Uniform double in [0,1) with 53 random bits from one Philox block.
__host__ __device__ inline double philox_uniform(unsigned long long seed, uint32_t c0,
                                                 uint32_t c1, uint32_t c2, uint32_t c3) {
  uint32_t c[4] = {c0, c1, c2, c3};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  const uint64_t m = ((uint64_t)(c[0] >> 5) << 26) | (uint64_t)(c[1] >> 6);
  return (double)m * 0x1.0p-53;
}

// Philox counter domains (top bits of the fourth word, run id below).
enum : uint32_t { DOM_INIT = 1u, DOM_PERTURB = 2u, DOM_SYSTEMATIC = 3u, DOM_FIELD = 4u };

// ---- drand48 (POSIX 48-bit LCG), with jump-ahead ----------------------------
constexpr uint64_t D48_A = 0x5DEECE66DULL, D48_C = 0xBULL, D48_MASK = (1ULL << 48) - 1;
__host__ __device__ inline uint64_t d48_skip(uint64_t x, uint64_t n) {
  uint64_t am = 1, cm = 0, a = D48_A, c = D48_C;
  while (n) {
    if (n & 1) {
      am = (am * a) & D48_MASK;
      cm = (cm * a + c) & D48_MASK;
    }
    c = ((a + 1) * c) & D48_MASK;
    a = (a * a) & D48_MASK;
    n >>= 1;
  }
  return (am * x + cm) & D48_MASK;
}
__host__ __device__ inline uint64_t d48_next(uint64_t x) { return (D48_A * x + D48_C) & D48_MASK; }
__host__ __device__ inline double d48_value(uint64_t x) { return (double)x * 0x1.0p-48; }

// ---- glibc rand() emulation: additive feedback r_n = r_{n-3} + r_{n-31} ----
struct GlibcRand {
  uint32_t r[34];
  int i;
  int pad_;
};
__host__ __device__ inline int32_t glibc_rand_next(GlibcRand &s) {
  const uint32_t a = s.r[(s.i + 3) % 34];
  const uint32_t b = s.r[(s.i + 31) % 34];
  const uint32_t v = a + b;
  s.r[s.i] = v;
  s.i = (s.i + 1) % 34;
  return (int32_t)(v >> 1);
}
inline void glibc_srand(GlibcRand &s, uint32_t seed) {
  uint32_t r[344];
  if (seed == 0) seed = 1;
  r[0] = seed;
  for (int i = 1; i < 31; i++) {
    int64_t v = (16807LL * (int64_t)(int32_t)r[i - 1]) % 2147483647LL;
    if (v < 0) v += 2147483647LL;
    r[i] = (uint32_t)v;
  }
  for (int i = 31; i < 34; i++) r[i] = r[i - 31];
  for (int i = 34; i < 344; i++) r[i] = r[i - 31] + r[i - 3];
  for (int i = 0; i < 34; i++) s.r[i] = r[310 + i];
  s.i = 0;
}

}  // namespace clbm
