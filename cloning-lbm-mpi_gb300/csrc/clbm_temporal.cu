// clbm_temporal.cu -- FP32 interval kernel with every clone resident on chip.
//
// One thread-block cluster per clone: the clone's H rows are split into CS
// bands of R = H/CS rows, each band in one CTA's shared memory (9 planes of
// R*W floats).  The T steps of the interval run without touching HBM except
// for the drag terms: P_0 is loaded once, S_T stored once.
//
// In-place update ("AA" pattern): one buffer A holds, alternately,
//   after a local step:  A[n][opp k] = P(n,k)        (post-collision, own node)
//   after a gather step: A[m][k]     = S_next(m,k)   (streamed, natural order)
// Step t with t even is a gather step: S(n,k) = A[n - c_k][opp k], or on a
// bounced slot A[n][k] (= P(n, opp k)); the collided P(n,k) is pushed to
// A[n + c_k][k], or to A[n][opp k] when slot (n, opp k) bounces back.  Step
// t odd is a local step: S(n,k) = A[n][k], P(n,k) -> A[n][opp k].  In both,
// the nine slots a node reads are exactly the nine it writes and no other
// node touches them, so a step needs no barrier inside; one cluster barrier
// separates steps.  These are the pull rules of clbm_step.cu (the reference's
// collide / push-stream / bounce-back / reset / swap sequence,
// src/mpi_LBM_GK_pops_perturb.cpp:426-443), so results are bit-identical to
// the streaming kernel.  Neighbours across a band edge are read and written
// in the adjacent CTA's shared memory (distributed shared memory).
#include <cooperative_groups.h>

#include "clbm_internal.h"
#include "clbm_physics.cuh"

namespace cg = cooperative_groups;

namespace clbm {

template <int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) k_temporal_f32(TemporalArgs a) {
  // A[node * 9 + k]: a node's nine values together (stride 9 words: no bank
  // conflicts across a warp), so every access is a base register plus an
  // immediate offset
  extern __shared__ float A[];
  cg::cluster_group cluster = cg::this_cluster();
  const int cs = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const RunDev &R = a.rd;
  const int clone = blockIdx.x / cs;
  const int W = R.W, H = R.H;
  const int rows = H / cs, row0 = rank * rows;
  const int nb = rows * W;
  float *prev = rank > 0 ? cluster.map_shared_rank(A, rank - 1) : A;
  float *next = rank + 1 < cs ? cluster.map_shared_rank(A, rank + 1) : A;
  const long long plane = R.plane;
  const long long cb = R.pop_base + (long long)clone * 9 * plane;
  const float *src = a.src + cb;
  float *dst = a.dst + cb;
  // P_0 into the "after a local step" layout
  for (int i = threadIdx.x; i < nb; i += THREADS) {
    const long long n = (long long)row0 * W + i;
#pragma unroll
    for (int k = 0; k < 9; k++) A[i * 9 + opp_of(k)] = src[k * plane + n];
  }
  // bulk[j]: the whole warp's node j is away from band edges, walls and the
  // square, so all its neighbours are in this CTA and nothing bounces back
  const int npt = (nb + THREADS - 1) / THREADS;
  unsigned bulk_bits = 0;
  for (int j = 0; j < npt && j < 32; j++) {
    const int i = threadIdx.x + j * THREADS;
    const int ly = (int)__umulhi((unsigned)i, R.div_w), x = i - ly * W, y = row0 + ly;
    const bool in_box = x >= R.xmin && x <= R.xmax && y >= R.ymin && y <= R.ymax;
    const bool ok = i >= nb || !(in_box || y == 0 || y == H - 1 || (cs > 1 && (ly == 0 || ly == rows - 1)));
    if (__all_sync(0xffffffffu, ok)) bulk_bits |= 1u << j;
  }
  const int rowstep = W * 9;  // one row in A, in words
  cluster.sync();
  for (int t = 0; t < a.steps; t++) {
    const bool gather = (t & 1) == 0, last = t == a.steps - 1;
    float *terms = a.terms + (long long)t * a.term_slab + R.term_base;
    for (int j = 0; j < npt; j++) {
      const int i = threadIdx.x + j * THREADS;
      if (i >= nb) continue;
      const int ly = (int)__umulhi((unsigned)i, R.div_w), x = i - ly * W, y = row0 + ly;
      const bool bulk = j < 32 && ((bulk_bits >> j) & 1u);
      // source / target columns: x-1 and x+1 with the periodic wrap
      const int cm = (x == 0 ? i + W - 1 : i - 1) * 9;
      const int c0 = i * 9;
      const int cp = (x == W - 1 ? i - (W - 1) : i + 1) * 9;
      float S[9];
      int mask = 0;
      bool in_box = false;
      if (bulk) {
        if (gather) {
          // S(n,k) = A[n - c_k][opp k]
          S[0] = A[c0 + 0];
          S[1] = A[cm + 3];
          S[2] = A[c0 - rowstep + 4];
          S[3] = A[cp + 1];
          S[4] = A[c0 + rowstep + 2];
          S[5] = A[cm - rowstep + 7];
          S[6] = A[cp - rowstep + 8];
          S[7] = A[cp + rowstep + 5];
          S[8] = A[cm + rowstep + 6];
        } else {
#pragma unroll
          for (int k = 0; k < 9; k++) S[k] = A[c0 + k];
        }
      } else {
        in_box = x >= R.xmin && x <= R.xmax && y >= R.ymin && y <= R.ymax;
        mask = (in_box || y == 0 || y == H - 1) ? bounce_mask(R, x, y) : 0;
        if (mask & 512) {  // inside the square
          if (last) {
            const long long n = (long long)y * W + x;
#pragma unroll
            for (int k = 0; k < 9; k++) dst[k * plane + n] = 0.0f;
          }
          continue;
        }
#pragma unroll
        for (int k = 0; k < 9; k++) {
          if (!gather || ((mask >> k) & 1)) {
            S[k] = A[c0 + k];
          } else {
            const int cx = cx_of(k), cy = cy_of(k);
            const int sxc = cx == 1 ? cm : (cx == -1 ? cp : c0);  // column, row ly
            const int sl = ly - cy;                                 // source row, band-local
            const float *base = sl < 0 ? prev : (sl >= rows ? next : A);
            const int roff = sl < 0 ? (rows - 1 - ly) * rowstep : (sl >= rows ? -ly * rowstep : -cy * rowstep);
            S[k] = base[sxc + roff + opp_of(k)];
          }
        }
        if (in_box) store_drag_terms<false>(R, S, x, y, clone, terms);
      }
      if (last) {
        const long long n = (long long)y * W + x;
        float d = 0.f;
#pragma unroll
        for (int k = 0; k < 9; k++) {
          dst[k * plane + n] = S[k];
          d += S[k];
        }
        if (!(d > -1.0f)) atomicOr(a.err, (unsigned)ERR_BAD_DENSITY);
        continue;
      }
      float beta = R.f_beta;
      if (R.field_mode && t + 1 < R.field_steps && a.maps)
        beta *= 1.0f + R.f_field_eps * a.maps[R.map_base + (long long)clone * R.nodes + (long long)y * W + x];
      float P[9];
      const float drho = collide_f32_pairs(S, P, beta, R.f_omega, R.f_cforce);
      if (!(drho > -1.0f)) atomicOr(a.err, (unsigned)ERR_BAD_DENSITY);
      if (bulk) {
        if (gather) {
          // P(n,k) -> A[n + c_k][k]
          A[c0 + 0] = P[0];
          A[cp + 1] = P[1];
          A[c0 + rowstep + 2] = P[2];
          A[cm + 3] = P[3];
          A[c0 - rowstep + 4] = P[4];
          A[cp + rowstep + 5] = P[5];
          A[cm + rowstep + 6] = P[6];
          A[cm - rowstep + 7] = P[7];
          A[cp - rowstep + 8] = P[8];
        } else {
#pragma unroll
          for (int k = 0; k < 9; k++) A[c0 + opp_of(k)] = P[k];
        }
      } else {
#pragma unroll
        for (int k = 0; k < 9; k++) {
          const int ok = opp_of(k);
          if (!gather || ((mask >> ok) & 1)) {
            A[c0 + ok] = P[k];
          } else {
            const int cx = cx_of(k), cy = cy_of(k);
            const int tx = cx == 1 ? (x == W - 1 ? 0 : x + 1) : (cx == -1 ? (x == 0 ? W - 1 : x - 1) : x);
            const int ty = y + cy;
            if (ty < 0 || ty >= H) continue;
            if (tx > R.xmin && tx < R.xmax && ty > R.ymin && ty < R.ymax) continue;  // into the square
            const int txc = cx == 1 ? cp : (cx == -1 ? cm : c0);
            const int tl = ly + cy;
            float *base = tl < 0 ? prev : (tl >= rows ? next : A);
            const int roff = tl < 0 ? (rows - 1 - ly) * rowstep : (tl >= rows ? -ly * rowstep : cy * rowstep);
            base[txc + roff + k] = P[k];
          }
        }
      }
    }
    cluster.sync();
  }
}

struct TemporalVariant {
  int threads;
  void (*fn)(TemporalArgs);
};

static const TemporalVariant kTemporal[] = {
    {1024, k_temporal_f32<1024, 1>}, {512, k_temporal_f32<512, 2>}, {256, k_temporal_f32<256, 4>}};

int temporal_variant_count() { return (int)(sizeof(kTemporal) / sizeof(kTemporal[0])); }

// Launch one run's interval with cluster size cs (H % cs == 0); returns
// cudaErrorInvalidConfiguration when the band does not fit in shared memory.
cudaError_t launch_temporal(const TemporalArgs &a, int cs, int variant, int nclones, int W, int H,
                            cudaStream_t s) {
  if (variant < 0 || variant >= temporal_variant_count() || cs < 1 || H % cs) return cudaErrorInvalidValue;
  const TemporalVariant &v = kTemporal[variant];
  const size_t smem = sizeof(float) * 9 * (size_t)(H / cs) * W;
  if (smem > 227 * 1024) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaFuncSetAttribute(v.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (cs > 8) {
    e = cudaFuncSetAttribute(v.fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cs * nclones);
  cfg.blockDim = dim3(v.threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, v.fn, a);
}

// Whether the cluster shape can be resident at all (occupancy query, no launch).
int temporal_max_clusters(int cs, int variant, int W, int H) {
  if (variant < 0 || variant >= temporal_variant_count() || cs < 1 || H % cs) return 0;
  const TemporalVariant &v = kTemporal[variant];
  const size_t smem = sizeof(float) * 9 * (size_t)(H / cs) * W;
  if (smem > 227 * 1024) return 0;
  if (cudaFuncSetAttribute(v.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return 0;
  if (cs > 8 && cudaFuncSetAttribute(v.fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
    return 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cs * 64);
  cfg.blockDim = dim3(v.threads);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, (void *)v.fn, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

}  // namespace clbm
