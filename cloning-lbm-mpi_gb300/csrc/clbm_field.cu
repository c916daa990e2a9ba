// clbm_field.cu -- Gaussian random body-force fields of the forcing variant,
// one per clone per interval, on the device.
//
// The reference draws each field by circulant embedding
// (src/perturbation_routines/generate_random_field.cpp:9-181): embed the
// covariance c(dx,dy) = exp(-(dx^2+dy^2)/(2 sigma^2)) (covariance_fctn.cpp:3-10)
// in an M x M circulant (M = 2n-1), take its spectrum lambda = FFT2(G)/M^2,
// multiply sqrt(lambda) by complex N(0,1) draws and FFT2 again; the real part
// of the top-left n x n block is the field (map index y + Dy*x, :169-178).
// Here the domain is W x H (M1 = 2W-1, M2 = 2H-1) and, because only the W x H
// block is kept, the second transform is evaluated as two dense contractions
// instead of a full FFT:
//   stage 1  Y[x][b]   = sum_a  w1^(a x) s[a][b] Z[a][b]      x < W, b < M2
//   stage 2  map[x][y] = Re sum_b Y[x][b] w2^(b y)            y < H
// with w = exp(-2 pi i / M) (FFTW_FORWARD's sign), s = sqrt(max(lambda, 0))
// computed once per run on the host, and Z drawn from Philox4x32-10 by
// Box-Muller.  The field is stored as FP32 in the populations' node order
// y*W + x.
//
// Stage 1 carries most of the arithmetic (83 % of the multiply-adds for the
// reference's sigma = 32 on a 256 x 64 lattice) and runs on the tensor cores
// (tcgen05, TF32 operands, FP32 accumulation in tensor memory): per clone a
// real GEMM D = A B with
//   rows    m = (part, x): Re Y[x] for m < W, Im Y[x] for W <= m < 2W
//   K       k = 2a + q:    q = 0 the real, q = 1 the imaginary part of s Z[a]
//   columns n = b
//   A[(0,x)][(a,0)] = cos t, A[(0,x)][(a,1)] = sin t,
//   A[(1,x)][(a,0)] = -sin t, A[(1,x)][(a,1)] = cos t,  t = 2 pi (a x mod M1) / M1
// (w1^(a x) = cos t - i sin t).  A is the same for every clone: it is built
// once per run on the host, rounded to TF32, and stored in global memory as
// the shared-memory image the tensor core reads (K-major, no swizzle: 8-row x
// 16-byte core matrices, the K-adjacent ones 128 B apart, the row-adjacent
// ones 1024 B apart), one contiguous block per 32-wide K chunk, so that one
// bulk asynchronous copy stages a chunk.  B is drawn by the CTA's threads
// straight into shared memory in the same layout; a chunk of B is generated
// while the tensor core multiplies the previous one (two buffers, mbarrier
// hand-off).  The four 128-row tiles of a pass accumulate in 4 x 128 columns
// of tensor memory.  TF32 keeps 11 significant bits of the operands; the
// field's covariance tests bound the effect.
//
// Only the embedding's significant modes enter: lambda is separable, and the
// rows a and columns b whose 1-D eigenvalue lies below 1e-16 of the largest
// are left out (their amplitudes are below 1e-8 of the largest; together they
// move the field by under 3e-6 of its RMS).  The sums over a and b above run
// over the kept lists; every kept mode draws its normal from the same Philox
// counter (a M2 + b, clone, interval, run) as in the full transform.  For the
// reference's sigma = 32 on a 256 x 64 lattice this keeps 158 of 511 rows and
// all 127 columns (the periodised Gaussian is wide against the 127-column
// period).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "clbm_internal.h"

namespace clbm {

__device__ __forceinline__ int field_run(const RunDev *runs, int nruns, int g) {
  int r = 0;
  while (r + 1 < nruns && g >= runs[r + 1].clone_base) r++;
  return r;
}

namespace tc {
constexpr int THREADS = 512;
constexpr int KC = 32;              // K elements (tf32) per chunk
constexpr int NT = 128;             // columns (b) per tile
constexpr int MT = 128;             // rows per tile
constexpr int TILES = 4;            // tiles per pass: 4 x 128 columns of tensor memory
constexpr int TILE_FLOATS = MT * KC;            // 4096 floats = 16 KB per tile and chunk
constexpr int A_BYTES = TILES * TILE_FLOATS * 4;  // 64 KB
constexpr int B_BYTES = NT * KC * 4;              // 16 KB
constexpr int SMEM = 2 * A_BYTES + 2 * B_BYTES + 64;
constexpr unsigned TMEM_COLS = 512;
constexpr long long WAIT_LIMIT = 1LL << 22;  // try_wait polls before a wait gives up

// element (row r, k) of a 128-row x 32-k operand tile, in floats: core
// matrix (r/8, k/4) of 32 floats (128 B), row r%8 of 4 floats in it
__host__ __device__ inline int tile_index(int r, int k) {
  return ((r >> 3) * 8 + (k >> 2)) * 32 + (r & 7) * 4 + (k & 3);
}

// shared-memory matrix descriptor: start address, leading-dimension (K)
// byte offset 128, stride-dimension (row group) byte offset 1024, the
// descriptor version bit, no swizzle
__device__ __forceinline__ unsigned long long smem_desc(unsigned addr) {
  return (unsigned long long)((addr >> 4) & 0x3FFFu) | ((unsigned long long)(128u >> 4) << 16) |
         ((unsigned long long)(1024u >> 4) << 32) | (1ull << 46);
}

// instruction descriptor: D FP32, A and B TF32, both K-major, M = 128, N = n
// (a multiple of 16 up to 256)
__device__ __forceinline__ unsigned idesc(int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((unsigned)(n >> 3) << 17) | ((unsigned)(MT >> 4) << 24);
}

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// wait for the completion of the barrier's phase of this parity; false when
// the bounded number of polls ran out
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
  for (long long i = 0; i < WAIT_LIMIT; i++) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}
__device__ __forceinline__ void bulk_load(unsigned dst, const void *src, unsigned bytes, unsigned bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void mma_tf32(unsigned d, unsigned long long a, unsigned long long b, unsigned id,
                                         unsigned acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(d),
      "l"(a), "l"(b), "r"(id), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(unsigned bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ float tf32_round(float v) {
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
  return __uint_as_float(r);
}
// 16 consecutive accumulator columns of the warp's 32 lanes, one row per thread
__device__ __forceinline__ void tmem_ld16(unsigned taddr, float v[16]) {
  unsigned r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
}  // namespace tc

// Stage 1 on the tensor cores, one CTA per clone: every (pass of four 128-row
// tiles, column tile of up to 128 kept columns) unit runs the whole K loop in
// 32-wide chunks (16 kept rows a each).
__global__ void __launch_bounds__(tc::THREADS, 1) k_field_stage1_tc(FieldArgs a) {
  using namespace tc;
  extern __shared__ __align__(1024) unsigned char smem[];
  const int g = blockIdx.x;
  const int r = field_run(a.runs, a.nruns, g);
  const RunDev &R = a.runs[r];
  if (R.field_mode == 0) return;
  const int W = R.W, M2 = R.M2, na = R.fna, nb = R.fnb;
  const int clone = g - R.clone_base;
  const int interval = a.state[r].interval;
  const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
  const int *alist = a.flist + R.flist_base, *blist = alist + na;
  float *A_s[2] = {(float *)smem, (float *)(smem + A_BYTES)};
  float *B_s[2] = {(float *)(smem + 2 * A_BYTES), (float *)(smem + 2 * A_BYTES + B_BYTES)};
  unsigned long long *bars = (unsigned long long *)(smem + 2 * A_BYTES + 2 * B_BYTES);
  unsigned &tmem_base_s = *(unsigned *)(bars + 4);
  // set only before a __syncthreads and read only after it: every thread
  // takes the same branch on it
  int &abort_s = *(int *)(bars + 5);
  const unsigned full_a[2] = {smem_u32(&bars[0]), smem_u32(&bars[1])};
  const unsigned mma_done[2] = {smem_u32(&bars[2]), smem_u32(&bars[3])};
  if (tid == 0) {
    for (int i = 0; i < 4; i++) mbar_init(smem_u32(&bars[i]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_s = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const unsigned tmem = tmem_base_s;
  const float *spec = a.spec + R.spec_base;
  const float *dft = a.dft + R.fa_base;
  const int nbp = field_y_pitch(nb);  // row pitch of Y
  float *Yr = (float *)(a.ybuf + R.y_base) + (long long)clone * 2 * W * nbp, *Yi = Yr + (long long)W * nbp;
  const int ntiles_m = R.f_mpad / MT, passes = (ntiles_m + TILES - 1) / TILES;
  const int ntiles_n = (nb + NT - 1) / NT, nchunks = R.f_kchunks;
  int gc = 0;          // chunks issued by this CTA so far (buffer and mbarrier phase)
  bool ok = true;
  for (int unit = 0; unit < passes * ntiles_n; unit++) {
    const int pass = unit / ntiles_n, nt = unit % ntiles_n;
    const int tiles = min(TILES, ntiles_m - pass * TILES);
    const int ncols = min(NT, nb - nt * NT), nmma = (ncols + 15) & ~15;  // MMA N: multiple of 16
    const unsigned id = idesc(nmma);
    const float *dft_pass = dft + (long long)pass * TILES * nchunks * TILE_FLOATS;
    for (int c = 0; c < nchunks; c++, gc++) {
      const int buf = gc & 1, use = gc >> 1;
      // the buffer is free once the MMAs of its previous chunk completed
      if (gc >= 2 && !mbar_wait(mma_done[buf], (use - 1) & 1)) ok = false;
      if (tid == 0 && ok) {
        const unsigned bytes = (unsigned)tiles * TILE_FLOATS * 4;
        mbar_expect_tx(full_a[buf], bytes);
        bulk_load(smem_u32(A_s[buf]), dft_pass + (long long)c * tiles * TILE_FLOATS, bytes, full_a[buf]);
      }
      // B chunk: rows n (kept column), K = 2 j + q for kept rows j in
      // [16c, 16c + 16), one complex draw per (a, b) = (alist[j], blist[n])
      // written as the pair (k, k + 1).  The thread's sqrt(lambda) loads are
      // issued first; the draws do not depend on them (a zero amplitude or a
      // padding slot scales the draw to zero).
      float *B = B_s[buf];
      constexpr int PER = 16 * NT / THREADS;
      float sv[PER];
#pragma unroll
      for (int j = 0; j < PER; j++) {
        const int d = tid + j * THREADS, jr = c * 16 + d / nmma, n = d % nmma, jc = nt * NT + n;
        sv[j] = (d < 16 * nmma && jr < na && n < ncols) ? __ldg(spec + (long long)jr * nb + jc) : 0.0f;
      }
#pragma unroll
      for (int j = 0; j < PER; j++) {
        const int d = tid + j * THREADS;
        if (d >= 16 * nmma) break;
        const int al = d / nmma, n = d % nmma, jr = c * 16 + al, jc = nt * NT + n;
        const int av = jr < na ? alist[jr] : 0, b = n < ncols ? blist[jc] : 0;
        uint32_t ctr[4] = {(uint32_t)(av * M2 + b), (uint32_t)clone, (uint32_t)interval,
                           (R.run_id << 4) | DOM_FIELD};
        philox4x32_10(ctr, (uint32_t)R.seed, (uint32_t)(R.seed >> 32));
        const float u1 = ((float)ctr[0] + 1.0f) * 0x1.0p-32f;  // (0, 1]
        const float u2 = (float)ctr[1] * 0x1.0p-32f;           // [0, 1)
        const float rad = sv[j] * sqrtf(-2.0f * logf(u1));
        float sn, cs;
        sincospif(2.0f * u2, &sn, &cs);
        *(float2 *)(B + tile_index(n, 2 * al)) = make_float2(tf32_round(rad * cs), tf32_round(rad * sn));
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // B visible to the tensor core
      if (!ok) abort_s = 1;
      __syncthreads();
      if (abort_s) break;
      if (tid == 0) {
        if (!mbar_wait(full_a[buf], use & 1)) {
          ok = false;  // published at the next check
        } else {
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const unsigned a0 = smem_u32(A_s[buf]), b0 = smem_u32(B_s[buf]);
          for (int t = 0; t < tiles; t++)
#pragma unroll
            for (int ks = 0; ks < KC / 8; ks++)
              mma_tf32(tmem + t * NT, smem_desc(a0 + t * TILE_FLOATS * 4 + ks * 256), smem_desc(b0 + ks * 256), id,
                       (c > 0 || ks > 0) ? 1u : 0u);
          mma_commit(mma_done[buf]);
        }
      }
    }
    if (!ok) abort_s = 1;
    __syncthreads();
    if (abort_s) break;
    // every MMA of the unit has completed once its last chunk's commit has
    if (!mbar_wait(mma_done[(gc - 1) & 1], ((gc - 1) >> 1) & 1)) abort_s = 1;
    __syncthreads();
    if (abort_s) break;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // accumulators -> Y: warp w reads lanes 32 (w % 4) .. + 31 (rows) and
    // columns 32 (w / 4) .. + 31 of each tile
    const int q = warp % 4, h = warp / 4;
    static_assert(THREADS == 512, "16 warps: 4 lane quarters x 4 column quarters");
    for (int t = 0; t < tiles; t++) {
      const int m = (pass * TILES + t) * MT + 32 * q + lane;
      float *dst = m < W ? Yr + (long long)m * nbp : (m < 2 * W ? Yi + (long long)(m - W) * nbp : nullptr);
      // columns of this tile inside the padded row (the padding takes the
      // accumulators of the empty columns, zeros)
      const int ncols_p = min(NT, nbp - nt * NT);
#pragma unroll
      for (int j = 0; j < 2; j++) {
        const int n0 = 32 * h + 16 * j;
        float v[16];
        tmem_ld16(tmem + ((unsigned)(32 * q) << 16) + t * NT + n0, v);
        if (dst) {
#pragma unroll
          for (int i = 0; i < 4; i++)
            if (n0 + 4 * i + 3 < ncols_p)
              *(float4 *)(dst + nt * NT + n0 + 4 * i) = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();  // accumulators read before the next unit overwrites them
  }
  if (abort_s) {
    // a wait gave up: flag it, let every MMA this CTA issued finish (bounded)
    if (tid == 0) {
      atomicOr(a.err, (unsigned)ERR_TIMEOUT);
      if (gc > 0) mbar_wait(mma_done[(gc - 1) & 1], ((gc - 1) >> 1) & 1);
    }
    __syncthreads();
  }
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

// Stage 2: map[x][y] = sum over the kept columns j of Re Y[x][j] w2^(b_j y)
// = Yr cos + Yi sin (w2^(b y) = cos - i sin).  A CTA computes a 64 x 64 tile
// of outputs, each thread a 4 x 4 register block (x = x0 + tx + 16 i,
// y = y0 + ty + 16 j): per kept column it reads four Y values and four
// twiddles from shared memory for sixteen outputs.  Every output still sums
// the kept columns in their order with the same fused multiply-adds, so the
// field is bit-identical to a one-output-per-thread loop.
constexpr int F2_T = 64;            // outputs per tile side
constexpr int F2_KB = 32;           // kept columns per staged chunk
constexpr int F2_LD = F2_T + 1;     // staging row length (float2): no bank conflicts on the transposed stores
constexpr int F2_THREADS = 256;     // 16 x 16 threads, 4 x 4 outputs each

__global__ void __launch_bounds__(F2_THREADS) k_field_stage2(FieldArgs a) {
  extern __shared__ float2 sh[];
  const int g = blockIdx.y;
  const int r = field_run(a.runs, a.nruns, g);
  const RunDev &R = a.runs[r];
  if (R.field_mode == 0) return;
  const int W = R.W, H = R.H, M2 = R.M2, nb = R.fnb;
  const int tilesx = (W + F2_T - 1) / F2_T;
  const int tile = blockIdx.x;
  if (tile >= tilesx * ((H + F2_T - 1) / F2_T)) return;
  const int x0 = (tile % tilesx) * F2_T, y0 = (tile / tilesx) * F2_T;
  const int clone = g - R.clone_base;
  float2 *tw = sh;                    // M2 twiddles
  float2 *Ys = tw + M2;               // [F2_KB][F2_LD]: Y of the chunk's columns, x-major rows
  float2 *Bs = Ys + F2_KB * F2_LD;    // [F2_KB][F2_LD]: w2^(b y) of the chunk's columns
  const float2 *tw_g = a.twiddles + R.tw2_base;
  for (int i = threadIdx.x; i < M2; i += F2_THREADS) tw[i] = tw_g[i];
  const int *blist = a.flist + R.flist_base + R.fna;
  const int nbp = field_y_pitch(nb);
  const float *Y = (const float *)(a.ybuf + R.y_base) + (long long)clone * 2 * W * nbp;  // Re rows, then Im rows
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 0.f;
  for (int jb = 0; jb < nb; jb += F2_KB) {
    __syncthreads();  // the previous chunk is consumed (and, first time, tw is loaded)
    for (int i = threadIdx.x; i < F2_T * F2_KB; i += F2_THREADS) {
      const int xi = x0 + i / F2_KB, k = i % F2_KB, j = jb + k;  // coalesced along j in Y
      Ys[k * F2_LD + i / F2_KB] = (xi < W && j < nb) ? make_float2(Y[(long long)xi * nbp + j], Y[(long long)(W + xi) * nbp + j])
                                                     : make_float2(0.f, 0.f);
    }
    for (int i = threadIdx.x; i < F2_T * F2_KB; i += F2_THREADS) {
      const int k = i / F2_T, yy = y0 + i % F2_T, j = jb + k;
      Bs[k * F2_LD + i % F2_T] =
          (j < nb && yy < H) ? tw[(int)(((unsigned)blist[j] * (unsigned)yy) % (unsigned)M2)] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int kmax = min(F2_KB, nb - jb);
    for (int k = 0; k < kmax; k++) {
      float2 v[4], t[4];
#pragma unroll
      for (int i = 0; i < 4; i++) v[i] = Ys[k * F2_LD + tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; j++) t[j] = Bs[k * F2_LD + ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(v[i].x, t[j].x, fmaf(-v[i].y, t[j].y, acc[i][j]));
    }
  }
  float *map = a.maps + R.map_base + (long long)clone * W * H;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const int y = y0 + ty + 16 * j;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int x = x0 + tx + 16 * i;
      if (x < W && y < H) map[(long long)y * W + x] = acc[i][j];
    }
  }
}

cudaError_t launch_fields(const FieldArgs &a, int total_clones, int max_w, int max_m1, int max_m2,
                          int max_tiles2, cudaStream_t s) {
  (void)max_w;
  (void)max_m1;
  // (set on every launch: the attribute belongs to the current device)
  cudaError_t e = cudaFuncSetAttribute(k_field_stage1_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM);
  if (e != cudaSuccess) return e;
  k_field_stage1_tc<<<total_clones, tc::THREADS, tc::SMEM, s>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const size_t sh2 = sizeof(float2) * ((size_t)max_m2 + 2 * F2_LD * F2_KB);
  dim3 g2(max_tiles2, total_clones);
  k_field_stage2<<<g2, F2_THREADS, sh2, s>>>(a);
  return cudaGetLastError();
}

// The stage-1 operand image of one run (see the head of this file), TF32
// values in FP32 containers, columns k = 2 j + q for the kept rows
// a = alist[j]: out must hold mpad * 32 * kchunks floats.
void build_field_dft_image(int W, int M1, const int *alist, int na, int mpad, int kchunks, float *out) {
  using namespace tc;
  const int ntm = mpad / MT;
  for (int m = 0; m < mpad; m++) {
    const int part = m < W ? 0 : (m < 2 * W ? 1 : -1);
    const int x = part == 0 ? m : m - W;
    const int tm = m / MT, pass = tm / TILES, t = tm % TILES, rr = m % MT;
    const int tiles = std::min(TILES, ntm - pass * TILES);
    float *base = out + (long long)pass * TILES * kchunks * TILE_FLOATS;
    for (int k = 0; k < kchunks * KC; k++) {
      const int j = k / 2, qi = k % 2;
      double v = 0.0;
      if (part >= 0 && j < na) {
        const double th = 2.0 * M_PI * (double)(((long long)alist[j] * x) % M1) / M1;
        const double c = std::cos(th), sn = std::sin(th);
        v = part == 0 ? (qi == 0 ? c : sn) : (qi == 0 ? -sn : c);
      }
      // round to TF32 (nearest, ties away from zero): 10 explicit mantissa bits
      float f = (float)v;
      unsigned u;
      memcpy(&u, &f, 4);
      u = (u + 0x1000u) & 0xFFFFE000u;
      memcpy(&f, &u, 4);
      const int c = k / KC;
      base[((long long)c * tiles + t) * TILE_FLOATS + tile_index(rr, k % KC)] = f;
    }
  }
}

}  // namespace clbm
