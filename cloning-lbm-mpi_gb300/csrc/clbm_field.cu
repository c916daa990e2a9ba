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
// with w = exp(-2 pi i / M) (FFTW_FORWARD's sign) read from twiddle tables in
// shared memory, s = sqrt(max(lambda, 0)) computed once per run on the host,
// and Z drawn inside stage 1 from Philox4x32-10 by Box-Muller.  The field is
// stored as FP32 in the populations' node order y*W + x.
#include "clbm_internal.h"

namespace clbm {

constexpr int F1_THREADS = 256;
constexpr int F1_BN = 8;   // b columns per CTA
constexpr int F1_KC = 32;  // a rows staged per chunk (F1_KC * F1_BN == F1_THREADS)
static_assert(F1_KC * F1_BN == F1_THREADS, "one staged value per thread");

__device__ __forceinline__ int field_run(const RunDev *runs, int nruns, int g) {
  int r = 0;
  while (r + 1 < nruns && g >= runs[r + 1].clone_base) r++;
  return r;
}

template <int RPT>
__global__ void __launch_bounds__(F1_THREADS) k_field_stage1(FieldArgs a) {
  extern __shared__ float2 sh[];
  const int g = blockIdx.y;
  const int r = field_run(a.runs, a.nruns, g);
  const RunDev &R = a.runs[r];
  const int b0 = blockIdx.x * F1_BN;
  if (R.field_mode == 0 || b0 >= R.M2) return;
  const int M1 = R.M1, M2 = R.M2, W = R.W;
  const int clone = g - R.clone_base;
  const int interval = a.state[r].interval;
  float2 *tw = sh;                 // M1 twiddles
  float2 *B = sh + M1;             // F1_KC x F1_BN staged values
  const float2 *tw_g = a.twiddles + R.tw1_base;
  for (int i = threadIdx.x; i < M1; i += F1_THREADS) tw[i] = tw_g[i];
  const float *spec = a.spec + R.spec_base;
  float2 acc[RPT][F1_BN];
#pragma unroll
  for (int q = 0; q < RPT; q++)
#pragma unroll
    for (int c = 0; c < F1_BN; c++) acc[q][c] = make_float2(0.f, 0.f);
  const int ka = threadIdx.x / F1_BN, cb = threadIdx.x % F1_BN;
  for (int a0 = 0; a0 < M1; a0 += F1_KC) {
    __syncthreads();
    {
      const int ai = a0 + ka, bi = b0 + cb;
      float2 v = make_float2(0.f, 0.f);
      if (ai < M1 && bi < M2) {
        const float s = spec[(long long)ai * M2 + bi];
        if (s != 0.f) {
          uint32_t ctr[4] = {(uint32_t)(ai * M2 + bi), (uint32_t)clone, (uint32_t)interval,
                             (R.run_id << 4) | DOM_FIELD};
          philox4x32_10(ctr, (uint32_t)R.seed, (uint32_t)(R.seed >> 32));
          const float u1 = ((float)ctr[0] + 1.0f) * 0x1.0p-32f;  // (0, 1]
          const float u2 = (float)ctr[1] * 0x1.0p-32f;           // [0, 1)
          const float rad = s * sqrtf(-2.0f * logf(u1));
          float sn, cs;
          sincospif(2.0f * u2, &sn, &cs);
          v = make_float2(rad * cs, rad * sn);
        }
      }
      B[ka * F1_BN + cb] = v;
    }
    __syncthreads();
    const int kmax = min(F1_KC, M1 - a0);
#pragma unroll
    for (int q = 0; q < RPT; q++) {
      const int x = threadIdx.x + q * F1_THREADS;
      if (x >= W) continue;
      int idx = (int)(((long long)a0 * x) % M1);
      for (int k = 0; k < kmax; k++) {
        const float2 t = tw[idx];
#pragma unroll
        for (int c = 0; c < F1_BN; c++) {
          const float2 bv = B[k * F1_BN + c];
          acc[q][c].x = fmaf(t.x, bv.x, fmaf(-t.y, bv.y, acc[q][c].x));
          acc[q][c].y = fmaf(t.x, bv.y, fmaf(t.y, bv.x, acc[q][c].y));
        }
        idx += x;
        if (idx >= M1) idx -= M1;
      }
    }
  }
  float2 *Y = a.ybuf + R.y_base + (long long)clone * W * M2;
#pragma unroll
  for (int q = 0; q < RPT; q++) {
    const int x = threadIdx.x + q * F1_THREADS;
    if (x >= W) continue;
#pragma unroll
    for (int c = 0; c < F1_BN; c++)
      if (b0 + c < M2) Y[(long long)x * M2 + b0 + c] = acc[q][c];
  }
}

constexpr int F2_TX = 16, F2_TY = 16, F2_KB = 64;

__global__ void __launch_bounds__(F2_TX *F2_TY) k_field_stage2(FieldArgs a) {
  extern __shared__ float2 sh[];
  const int g = blockIdx.y;
  const int r = field_run(a.runs, a.nruns, g);
  const RunDev &R = a.runs[r];
  if (R.field_mode == 0) return;
  const int W = R.W, H = R.H, M2 = R.M2;
  const int tilesx = (W + F2_TX - 1) / F2_TX;
  const int tile = blockIdx.x;
  if (tile >= tilesx * ((H + F2_TY - 1) / F2_TY)) return;
  const int x0 = (tile % tilesx) * F2_TX, y0 = (tile / tilesx) * F2_TY;
  const int clone = g - R.clone_base;
  float2 *tw = sh;             // M2 twiddles
  float2 *Ys = sh + M2;        // F2_TX x F2_KB
  const float2 *tw_g = a.twiddles + R.tw2_base;
  for (int i = threadIdx.x; i < M2; i += F2_TX * F2_TY) tw[i] = tw_g[i];
  const float2 *Y = a.ybuf + R.y_base + (long long)clone * W * M2;
  const int tx = threadIdx.x % F2_TX, ty = threadIdx.x / F2_TX;
  const int x = x0 + tx, y = y0 + ty;
  float acc = 0.f;
  for (int bb = 0; bb < M2; bb += F2_KB) {
    __syncthreads();
    for (int i = threadIdx.x; i < F2_TX * F2_KB; i += F2_TX * F2_TY) {
      const int xi = x0 + i / F2_KB, bi = bb + i % F2_KB;
      Ys[i] = (xi < W && bi < M2) ? Y[(long long)xi * M2 + bi] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    if (x < W && y < H) {
      const int kmax = min(F2_KB, M2 - bb);
      int idx = (int)(((long long)bb * y) % M2);
      for (int k = 0; k < kmax; k++) {
        const float2 t = tw[idx], v = Ys[tx * F2_KB + k];
        acc = fmaf(v.x, t.x, fmaf(-v.y, t.y, acc));
        idx += y;
        if (idx >= M2) idx -= M2;
      }
    }
  }
  if (x < W && y < H) a.maps[R.map_base + (long long)clone * W * H + (long long)y * W + x] = acc;
}

cudaError_t launch_fields(const FieldArgs &a, int total_clones, int max_w, int max_m1, int max_m2,
                          int max_tiles2, cudaStream_t s) {
  const size_t sh1 = sizeof(float2) * ((size_t)max_m1 + F1_KC * F1_BN);
  dim3 g1((max_m2 + F1_BN - 1) / F1_BN, total_clones);
  if (max_w <= F1_THREADS)
    k_field_stage1<1><<<g1, F1_THREADS, sh1, s>>>(a);
  else if (max_w <= 2 * F1_THREADS)
    k_field_stage1<2><<<g1, F1_THREADS, sh1, s>>>(a);
  else
    k_field_stage1<4><<<g1, F1_THREADS, sh1, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const size_t sh2 = sizeof(float2) * ((size_t)max_m2 + F2_TX * F2_KB);
  dim3 g2(max_tiles2, total_clones);
  k_field_stage2<<<g2, F2_TX * F2_TY, sh2, s>>>(a);
  return cudaGetLastError();
}

}  // namespace clbm
