// clbm_step.cu -- the batched stream-collide step and the kernels that prepare
// an interval (copy + perturbation + first collision), all over the
// structure-of-arrays population buffer of every clone of every run.
//
// Buffer semantics ("pull" scheme).  Between steps the buffer holds the
// POST-collision populations P of every fluid node.  Step t reads P_t,
// gathers the streamed state S_{t+1}(n,k) = P_t(n - c_k, k) -- or, where the
// reference bounces the slot back, the node's own P_t(n, opp k) -- resets
// square-interior nodes to w[k], evaluates the drag terms of S_{t+1} on the
// square perimeter, collides and writes P_{t+1}.  This is the reference's
// collide -> push-stream -> wall BB -> square BB -> interior reset -> swap
// -> drag sequence (src/mpi_LBM_GK_pops_perturb.cpp:426-445) with the time
// origin moved by half a step, so each node is read and written exactly once
// per step with aligned stores.  The last step of an interval writes S instead
// of P, because the cloning step and the perturbation act on S.
#include <cstdint>

#include "clbm_internal.h"
#include "clbm_physics.cuh"
#include "clbm_reseed.cuh"

namespace clbm {

__device__ __forceinline__ int find_run_by_block(const RunDev *runs, int nruns, int b) {
  int r = 0;
  while (r + 1 < nruns && b >= runs[r + 1].block_base) r++;
  return r;
}

struct NodeLoc {
  int run, clone, n, x, y;
  bool valid;
};

__device__ __forceinline__ NodeLoc locate(const RunDev *runs, int nruns) {
  NodeLoc L;
  const int b = blockIdx.x;
  L.run = find_run_by_block(runs, nruns, b);
  const RunDev &R = runs[L.run];
  const int local = b - R.block_base;
  L.clone = local / R.blocks_per_clone;
  const int tile = local - L.clone * R.blocks_per_clone;
  L.n = tile * blockDim.x + threadIdx.x;
  L.valid = L.n < R.nodes && L.clone < R.nclones;
  L.y = (int)__umulhi((unsigned)L.n, R.div_w);
  L.x = L.n - L.y * R.W;
  return L;
}

template <bool F64>
__device__ __forceinline__ bool density_ok(const pop_t<F64> S[9]) {
  if constexpr (F64) {
    double r = S[0];
#pragma unroll
    for (int k = 1; k < 9; k++) r += S[k];
    return r > 0.0;
  } else {
    float d = 0.f;
#pragma unroll
    for (int k = 0; k < 9; k++) d += S[k];
    return d > -1.0f;
  }
}

template <bool F64, bool LAST>
__global__ void __launch_bounds__(STEP_BLOCK) k_step(StepArgs a) {
  using T = pop_t<F64>;
  const NodeLoc L = locate(a.runs, a.nruns);
  if (!L.valid) return;
  const RunDev &R = a.runs[L.run];
  const long long plane = R.plane;
  const long long cbase = R.pop_base + (long long)L.clone * 9 * plane;
  const T *__restrict__ src = (const T *)a.src + cbase;
  T *__restrict__ dst = (T *)a.dst + cbase;
  const int x = L.x, y = L.y, n = L.n, W = R.W;

  const bool in_box = x >= R.xmin && x <= R.xmax && y >= R.ymin && y <= R.ymax;
  const int mask = (in_box || y == 0 || y == R.H - 1) ? bounce_mask(R, x, y) : 0;
  if (mask & 512) {
    // inside the square: reset to w[k] (stored shifted as 0 in FP32); its
    // post-collision values are never pulled by a fluid node
    if (LAST) {
#pragma unroll
      for (int k = 0; k < 9; k++) dst[k * plane + n] = F64 ? (T)w_of(k) : (T)0;
    }
    return;
  }
  const int xl = (x == 0) ? W - 1 : x - 1;
  const int xr = (x == W - 1) ? 0 : x + 1;
  const int row = y * W;
  T S[9];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const int cx = cx_of(k), cy = cy_of(k);
    const int sx = cx == 1 ? xl : (cx == -1 ? xr : x);
    const int srow = cy == 1 ? row - W : (cy == -1 ? row + W : row);
    const T *p = ((mask >> k) & 1) ? src + opp_of(k) * plane + n : src + k * plane + srow + sx;
    S[k] = __ldg(p);
  }
  if (in_box) {
    T *terms = (T *)a.terms + (long long)a.step * a.term_slab + R.term_base;
    store_drag_terms<F64>(R, S, x, y, L.clone, terms);
  }
  if (!density_ok<F64>(S)) atomicOr(a.err, (unsigned)ERR_BAD_DENSITY);
  if (LAST) {
#pragma unroll
    for (int k = 0; k < 9; k++) dst[k * plane + n] = S[k];
  } else {
    T P[9];
    collide_node<F64>(R, S, P, node_map(a.maps, R, L.clone, n, R.field_mode && a.step + 1 < R.field_steps));
#pragma unroll
    for (int k = 0; k < 9; k++) dst[k * plane + n] = P[k];
  }
}

// ---------------------------------------------------------------------------
// FP32 step, the hot kernel.  Grid: x = tile of BLOCK consecutive nodes,
// y = global clone index (no integer division to find the work).  Warps with
// no node on a wall row or in the square's bounding box (the bulk) take a
// path without any bounce-back selects; the decision is warp-uniform.
// Collision by opposite pairs (collide_f32_pairs).
template <int BLOCK>
__device__ __forceinline__ constexpr int tile_slot() {
  return BLOCK == 128 ? 0 : (BLOCK == 256 ? 1 : 2);
}

template <int BLOCK, int MINB, bool CS, bool LAST>
__global__ void __launch_bounds__(BLOCK, MINB) k_step_f32(StepArgs a) {
  constexpr int TS = tile_slot<BLOCK>();
  const int b = blockIdx.x;
  int r = 0;
  while (r + 1 < a.nruns && b >= a.runs[r + 1].tile_base[TS]) r++;
  const RunDev &R = a.runs[r];
  const unsigned local = (unsigned)(b - R.tile_base[TS]);
  const int clone = (int)__umulhi(local, R.tiles_div[TS]);
  const int tile = (int)local - clone * R.tiles[TS];
  const int n = tile * BLOCK + threadIdx.x;
  const int W = R.W, H = R.H;
  const bool valid = n < R.nodes;
  const int y = (int)__umulhi((unsigned)n, R.div_w);
  const int x = n - y * W;
  const bool in_box = x >= R.xmin && x <= R.xmax && y >= R.ymin && y <= R.ymax;
  const bool near = valid && (in_box || y == 0 || y == H - 1);
  const bool warp_near = __any_sync(0xffffffffu, near);
  if (!valid) return;
  const int plane = (int)R.plane;
  const long long cb = R.pop_base + (long long)clone * 9 * R.plane;
  const float *__restrict__ src = (const float *)a.src + cb;
  float *__restrict__ dst = (float *)a.dst + cb;
  const int xl = (x == 0) ? W - 1 : x - 1;
  const int xr = (x == W - 1) ? 0 : x + 1;
  const int row = y * W;
  int off[9];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const int cx = cx_of(k), cy = cy_of(k);
    const int sx = cx == 1 ? xl : (cx == -1 ? xr : x);
    const int srow = cy == 1 ? row - W : (cy == -1 ? row + W : row);
    off[k] = k * plane + srow + sx;
  }
  if (warp_near) {
    const int mask = near ? bounce_mask(R, x, y) : 0;
    if (mask & 512) {
      if (LAST) {
#pragma unroll
        for (int k = 0; k < 9; k++) dst[k * plane + n] = 0.0f;
      }
      return;
    }
#pragma unroll
    for (int k = 0; k < 9; k++)
      if ((mask >> k) & 1) off[k] = opp_of(k) * plane + n;
  }
  float S[9];
#pragma unroll
  for (int k = 0; k < 9; k++) S[k] = __ldg(src + off[k]);
  if (in_box) {
    float *terms = (float *)a.terms + (long long)a.step * a.term_slab + R.term_base;
    store_drag_terms<false>(R, S, x, y, clone, terms);
  }
  float P[9];
  float drho;
  if (LAST) {
    drho = 0.f;
#pragma unroll
    for (int k = 0; k < 9; k++) {
      P[k] = S[k];
      drho += S[k];
    }
  } else {
    const float *fm = (R.field_mode && a.step + 1 < R.field_steps && a.maps)
                          ? a.maps + R.map_base + (long long)clone * R.nodes + n
                          : nullptr;
    drho = collide_f32_run(R, S, P, fm, R.f_field_eps);
  }
  if (!(drho > -1.0f)) atomicOr(a.err, (unsigned)ERR_BAD_DENSITY);
#pragma unroll
  for (int k = 0; k < 9; k++) {
    if (CS)
      __stcs(dst + k * plane + n, P[k]);
    else
      dst[k * plane + n] = P[k];
  }
}

struct F32Variant {
  int block;
  void (*body)(StepArgs);
  void (*last)(StepArgs);
};

#define F32V(B, M, C) {B, k_step_f32<B, M, C, false>, k_step_f32<B, M, C, true>}
static const F32Variant kF32Variants[] = {
    F32V(256, 4, false), F32V(256, 5, false), F32V(256, 6, false), F32V(128, 8, false),
    F32V(128, 12, false), F32V(512, 2, false), F32V(256, 5, true), F32V(128, 12, true),
};
#undef F32V

int step_variant_count() { return (int)(sizeof(kF32Variants) / sizeof(kF32Variants[0])); }

int step_variant_block(int v) { return kF32Variants[v].block; }

cudaError_t launch_step(bool f64, bool last, const StepArgs &a, int blocks, cudaStream_t s,
                        int variant) {
  if (f64) {
    if (last)
      k_step<true, true><<<blocks, STEP_BLOCK, 0, s>>>(a);
    else
      k_step<true, false><<<blocks, STEP_BLOCK, 0, s>>>(a);
  } else {
    if (variant < 0 || variant >= step_variant_count()) variant = 0;
    const F32Variant &v = kF32Variants[variant];
    const int ts = v.block == 128 ? 0 : (v.block == 256 ? 1 : 2);
    const int grid = a.total_tiles[ts];
    if (last)
      v.last<<<grid, v.block, 0, s>>>(a);
    else
      v.body<<<grid, v.block, 0, s>>>(a);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Reseed: the first kernel of an interval.  Slot j takes its parent's state
// S(labels[j]) (the clone copy, pops driver :658-701), new clones are
// perturbed (:412-416: snapshot mix, generatePerturbedState.cpp:4-38, or the
// counter-based uniform noise), and the result is collided into P.
template <bool F64>
__global__ void __launch_bounds__(STEP_BLOCK) k_reseed(ReseedArgs a) {
  using T = pop_t<F64>;
  const NodeLoc L = locate(a.runs, a.nruns);
  if (!L.valid) return;
  const RunDev &R = a.runs[L.run];
  const int x = L.x, y = L.y, n = L.n;
  const bool solid = x > R.xmin && x < R.xmax && y > R.ymin && y < R.ymax;
  if (solid) return;  // post-collision values of interior nodes are never pulled
  T P[9];
  reseed_node<F64>(a, R, L.run, L.clone, x, y, n, P);
  T *dst = (T *)a.dst + R.pop_base + (long long)L.clone * 9 * R.plane;
#pragma unroll
  for (int k = 0; k < 9; k++) dst[k * R.plane + n] = P[k];
}

cudaError_t launch_reseed(bool f64, const ReseedArgs &a, int blocks, cudaStream_t s) {
  if (f64)
    k_reseed<true><<<blocks, STEP_BLOCK, 0, s>>>(a);
  else
    k_reseed<false><<<blocks, STEP_BLOCK, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Norms of the snapshot-mix perturbation (generatePerturbedState.cpp:22-31):
// |f|^2 of the parent state and |sum_q r_q snap_q|^2 over all 9*Dx*Dy values.
// Each block reduces its nodes in a fixed tree order into partials[block];
// the finalize kernel adds the blocks of a clone in order.  (The reference
// adds all values sequentially; the fixed tree order differs from it only in
// the rounding of the two norms.)
template <bool F64>
__global__ void __launch_bounds__(STEP_BLOCK)
    k_perturb_norms(const RunDev *runs, int nruns, const void *srcv, const int *labels,
                    const int *mark, const double *prefactors, const double *snaps,
                    double *partials) {
  using T = pop_t<F64>;
  __shared__ double red[2][STEP_BLOCK / 32];
  const NodeLoc L = locate(runs, nruns);
  const RunDev &R = runs[L.run];
  const int gclone = R.clone_base + L.clone;
  // whole block exits together (one clone per block)
  if (L.clone >= R.nclones || R.perturb_mode != 1 || !mark[gclone]) return;
  double n0 = 0.0, n1 = 0.0;
  if (L.n < R.nodes) {
    const int parent = labels[gclone];
    const long long plane = R.plane;
    const T *src = (const T *)srcv + R.pop_base + (long long)parent * 9 * plane;
    const double *pre = prefactors + (long long)gclone * MAX_SNAP;
#pragma unroll
    for (int k = 0; k < 9; k++) {
      const double f = F64 ? (double)src[k * plane + L.n] : w_of(k) + (double)src[k * plane + L.n];
      const double *sp = snaps + R.snap_base + (long long)k * plane + L.n;
      double mix = DMUL(pre[0], sp[0]);
      for (int q = 1; q < R.nsnap; q++) mix = DADD(mix, DMUL(pre[q], sp[(long long)q * 9 * plane]));
      n0 = DADD(n0, DMUL(f, f));
      n1 = DADD(n1, DMUL(mix, mix));
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    n0 = DADD(n0, __shfl_down_sync(0xffffffffu, n0, o));
    n1 = DADD(n1, __shfl_down_sync(0xffffffffu, n1, o));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][warp] = n0;
    red[1][warp] = n1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a0 = red[0][0], a1 = red[1][0];
    for (int i = 1; i < STEP_BLOCK / 32; i++) {
      a0 = DADD(a0, red[0][i]);
      a1 = DADD(a1, red[1][i]);
    }
    partials[2 * (long long)blockIdx.x] = a0;
    partials[2 * (long long)blockIdx.x + 1] = a1;
  }
}

__global__ void k_perturb_finalize(const RunDev *runs, int nruns, const int *mark,
                                   const double *prefactors, const double *partials,
                                   double *pert, int total_clones) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total_clones) return;
  int r = 0;
  while (r + 1 < nruns && g >= runs[r + 1].clone_base) r++;
  const RunDev &R = runs[r];
  if (!mark[g] || R.perturb_mode != 1) return;
  const int c = g - R.clone_base;
  const long long b0 = R.block_base + (long long)c * R.blocks_per_clone;
  double n0 = partials[2 * b0], n1 = partials[2 * b0 + 1];
  for (int t = 1; t < R.blocks_per_clone; t++) {
    n0 = DADD(n0, partials[2 * (b0 + t)]);
    n1 = DADD(n1, partials[2 * (b0 + t) + 1]);
  }
  n0 = __dsqrt_rn(n0);
  n1 = __dsqrt_rn(n1);
  const double weight = DDIV(n0, n1);
  const double *pre = prefactors + (long long)g * MAX_SNAP;
  double sum = pre[0];
  for (int q = 1; q < R.nsnap; q++) sum = DADD(sum, pre[q]);
  const double a = DADD(1.0, DMUL(DMUL(sum, R.eps), weight));
  pert[2 * g] = weight;
  pert[2 * g + 1] = DDIV(1., a);
}

cudaError_t launch_perturb_norms(bool f64, const RunDev *runs, int nruns, const void *src,
                                 const int *labels, const int *mark, const double *prefactors,
                                 const double *snaps, double *partials, double *pert,
                                 int blocks, int total_clones, cudaStream_t s) {
  if (f64)
    k_perturb_norms<true><<<blocks, STEP_BLOCK, 0, s>>>(runs, nruns, src, labels, mark,
                                                         prefactors, snaps, partials);
  else
    k_perturb_norms<false><<<blocks, STEP_BLOCK, 0, s>>>(runs, nruns, src, labels, mark,
                                                          prefactors, snaps, partials);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_perturb_finalize<<<(total_clones + 255) / 256, 256, 0, s>>>(runs, nruns, mark, prefactors,
                                                                 partials, pert, total_clones);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Synthetic initial state, the same arithmetic as the oracle's
// orc_init_equilibrium: feq(rho=1, u=(u0,0)) * (1 + noise (2u - 1)) in the
// fluid, w[k] inside the square; stored as the pre-collision state S.
template <bool F64>
__global__ void __launch_bounds__(STEP_BLOCK)
    k_init_equilibrium(const RunDev *runs, int nruns, int run, void *popv, double u0,
                       double noise, unsigned long long seed) {
  using T = pop_t<F64>;
  const RunDev &R = runs[run];
  const int clone = blockIdx.y;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= R.nodes || clone >= R.nclones) return;
  const int y = n / R.W, x = n - y * R.W;
  const bool solid = x > R.xmin && x < R.xmax && y > R.ymin && y < R.ymax;
  T *pop = (T *)popv + R.pop_base + (long long)clone * 9 * R.plane;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    double f;
    if (solid) {
      f = w_of(k);
    } else {
      const double eu = DMUL((double)cx_of(k), u0);
      const double feq = DMUL(w_of(k), DADD(DADD(DADD(1.0, DMUL(3.0, eu)), DMUL(DMUL(4.5, eu), eu)),
                                            DMUL(-1.5, DMUL(u0, u0))));
      const double u = philox_uniform(seed, aos_index(R, x, y, k), (uint32_t)clone, 0xFFFFFFFFu,
                                      (R.run_id << 4) | DOM_INIT);
      f = DMUL(feq, DADD(1.0, DMUL(noise, DSUB(DMUL(2.0, u), 1.0))));
    }
    pop[k * R.plane + n] = F64 ? (T)f : (T)(f - w_of(k));
  }
}

cudaError_t launch_init_equilibrium(bool f64, const RunDev *runs, int nruns, int run, void *pop,
                                    double u0, double noise, unsigned long long seed, int blocks,
                                    cudaStream_t s) {
  (void)blocks;
  RunDev h;
  cudaError_t e = cudaMemcpyAsync(&h, runs + run, sizeof(RunDev), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return e;
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return e;
  dim3 grid((h.nodes + 255) / 256, h.nclones);
  if (f64)
    k_init_equilibrium<true><<<grid, 256, 0, s>>>(runs, nruns, run, pop, u0, noise, seed);
  else
    k_init_equilibrium<false><<<grid, 256, 0, s>>>(runs, nruns, run, pop, u0, noise, seed);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Layout conversion between the reference's AoS FP64 files/arrays
// (k + 9*(y + Dy*x)) and the device SoA buffer (plane k, node y*Dx + x).
template <bool F64>
__global__ void k_aos_to_soa(const RunDev *runs, int run, int clone0, const double *aos,
                             void *popv) {
  using T = pop_t<F64>;
  const RunDev &R = runs[run];
  const int c = blockIdx.y;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;  // AoS node order: t = y + H*x
  if (t >= R.nodes) return;
  const int x = t / R.H, y = t - x * R.H;
  const double *src = aos + (long long)c * 9 * R.nodes + 9LL * t;
  T *dst = (T *)popv + R.pop_base + (long long)(clone0 + c) * 9 * R.plane + (long long)y * R.W + x;
#pragma unroll
  for (int k = 0; k < 9; k++) dst[k * R.plane] = F64 ? (T)src[k] : (T)(src[k] - w_of(k));
}

template <bool F64>
__global__ void k_soa_to_aos(const RunDev *runs, int run, int clone, const void *popv,
                             double *aos) {
  using T = pop_t<F64>;
  const RunDev &R = runs[run];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= R.nodes) return;
  const int x = t / R.H, y = t - x * R.H;
  const T *src = (const T *)popv + R.pop_base + (long long)clone * 9 * R.plane + (long long)y * R.W + x;
#pragma unroll
  for (int k = 0; k < 9; k++) aos[9LL * t + k] = F64 ? (double)src[k * R.plane] : w_of(k) + (double)src[k * R.plane];
}

__global__ void k_snaps_to_soa(const RunDev *runs, int run, const double *aos, double *snaps) {
  const RunDev &R = runs[run];
  const int q = blockIdx.y;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= R.nodes) return;
  const int x = t / R.H, y = t - x * R.H;
  const double *src = aos + (long long)q * 9 * R.nodes + 9LL * t;
  double *dst = snaps + R.snap_base + (long long)q * 9 * R.plane + (long long)y * R.W + x;
#pragma unroll
  for (int k = 0; k < 9; k++) dst[k * R.plane] = src[k];
}

// Macroscopic fields of a clone's pre-collision state in the reference's node
// order idx(x,y) = y + Dy*x: rho, the force-shifted ux = jx/rho + beta/(2 rho)
// and uy, as streamCollCompute.cpp:21-28 computes them before colliding
// (the fields write_fluid_vtk prints, write_vtk.cpp:38-49).
template <bool F64>
__global__ void k_macro(const RunDev *runs, int run, int clone, const void *popv, double *rho,
                        double *ux, double *uy) {
  using T = pop_t<F64>;
  const RunDev &R = runs[run];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;  // t = y + H*x
  if (t >= R.nodes) return;
  const int x = t / R.H, y = t - x * R.H;
  const T *src = (const T *)popv + R.pop_base + (long long)clone * 9 * R.plane + (long long)y * R.W + x;
  double f[9];
#pragma unroll
  for (int k = 0; k < 9; k++) f[k] = F64 ? (double)src[k * R.plane] : w_of(k) + (double)src[k * R.plane];
  const Moments64 m = moments_ref64(f);
  rho[t] = m.rho;
  ux[t] = DADD(DDIV(m.jx, m.rho), DDIV(DMUL(0.5, R.beta), m.rho));
  uy[t] = DDIV(m.jy, m.rho);
}

cudaError_t launch_macro(bool f64, const RunDev *runs, int run, int clone, int nodes, const void *pop,
                         double *rho, double *ux, double *uy, cudaStream_t s) {
  if (f64)
    k_macro<true><<<(nodes + 255) / 256, 256, 0, s>>>(runs, run, clone, pop, rho, ux, uy);
  else
    k_macro<false><<<(nodes + 255) / 256, 256, 0, s>>>(runs, run, clone, pop, rho, ux, uy);
  return cudaGetLastError();
}

// (nodes = W*H of the run, from the host copy of its descriptor)
cudaError_t launch_aos_to_soa(bool f64, const RunDev *runs, int run, int nodes, int clone0, int nclone,
                              const double *aos, void *pop, cudaStream_t s) {
  dim3 grid((nodes + 255) / 256, nclone);
  if (f64)
    k_aos_to_soa<true><<<grid, 256, 0, s>>>(runs, run, clone0, aos, pop);
  else
    k_aos_to_soa<false><<<grid, 256, 0, s>>>(runs, run, clone0, aos, pop);
  return cudaGetLastError();
}

cudaError_t launch_soa_to_aos(bool f64, const RunDev *runs, int run, int nodes, int clone, const void *pop,
                              double *aos, cudaStream_t s) {
  if (f64)
    k_soa_to_aos<true><<<(nodes + 255) / 256, 256, 0, s>>>(runs, run, clone, pop, aos);
  else
    k_soa_to_aos<false><<<(nodes + 255) / 256, 256, 0, s>>>(runs, run, clone, pop, aos);
  return cudaGetLastError();
}

cudaError_t launch_snaps_to_soa(const RunDev *runs, int run, int nodes, int nsnap, const double *aos,
                                double *snaps, cudaStream_t s) {
  dim3 grid((nodes + 255) / 256, nsnap);
  k_snaps_to_soa<<<grid, 256, 0, s>>>(runs, run, aos, snaps);
  return cudaGetLastError();
}

}  // namespace clbm
