// clbm_refops.cu -- function-level entry points: the reference's LBM
// functions on one clone in its own FP64 array-of-structures layout
// IDX(x,y,k) = k + 9*(y + Dy*x) (src/lbm_src/global.h:4), on device pointers,
// with the reference's operation order (bit-identical results).
#include <cstdio>
#include <mutex>

#include "../../include/clbm.h"
#include "clbm_physics.cuh"

namespace clbm {

struct GeomDev {
  int nx, ny, xmin, xmax, ymin, ymax;
};

__device__ __forceinline__ long long aos(const GeomDev &g, int x, int y, int k) {
  return k + 9LL * (y + (long long)g.ny * x);
}

// streamCollCompute.cpp:7-93: collide in place into fin, push to the periodic
// neighbour in fout, macroscopic fields of the pre-collision state.
__global__ void k_ref_stream_collide(GeomDev g, double *fin, double *fout, double *rho,
                                     double *ux, double *uy, double beta0, const double *map,
                                     double tau, double eps) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;  // t = y + ny*x
  if (t >= g.nx * g.ny) return;
  const int x = t / g.ny, y = t - x * g.ny;
  const double omega = DDIV(1., tau);
  const double om1 = DSUB(1.0, omega);
  const double cforce = DSUB(1.0, DMUL(0.5, omega));
  double beta = beta0;
  if (map) beta = DMUL(DADD(1.0, DMUL(eps, map[t])), beta0);
  double wcb[9];
#pragma unroll
  for (int k = 0; k < 9; k++) wcb[k] = DMUL(DMUL(w_of(k), cforce), beta);
  double f[9], post[9];
#pragma unroll
  for (int k = 0; k < 9; k++) f[k] = fin[aos(g, x, y, k)];
  double r, vx, vy;
  collide_ref64(f, post, beta, wcb, omega, om1, &r, &vx, &vy);
#pragma unroll
  for (int k = 0; k < 9; k++) {
    fin[aos(g, x, y, k)] = post[k];
    const int tx = (x + cx_of(k) + g.nx) % g.nx;
    const int ty = (y + cy_of(k) + g.ny) % g.ny;
    fout[aos(g, tx, ty, k)] = post[k];
  }
  if (ux) ux[t] = vx;
  if (uy) uy[t] = vy;
  if (rho) rho[t] = r;
}

// domain_noSlipWalls.cpp:6-22
__global__ void k_ref_walls(GeomDev g, double *fout, const double *fin) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= g.nx) return;
  const int top = g.ny - 1;
  const int up[3] = {2, 5, 6}, down[3] = {4, 7, 8};
#pragma unroll
  for (int i = 0; i < 3; i++) {
    fout[aos(g, x, top, down[i])] = fin[aos(g, x, top, opp_of(down[i]))];
    fout[aos(g, x, 0, up[i])] = fin[aos(g, x, 0, opp_of(up[i]))];
  }
}

// square.cpp:24-50 (the live _TEST variant); one thread per perimeter node
__global__ void k_ref_square(GeomDev g, double *fout, const double *fin) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int sx = g.xmax - g.xmin, sy = g.ymax - g.ymin;
  const int bottom[3] = {7, 4, 8}, top[3] = {5, 2, 6}, left[3] = {6, 3, 7}, right[3] = {8, 1, 5};
  if (i < sx - 1) {
    const int x = g.xmin + 1 + i;
#pragma unroll
    for (int q = 0; q < 3; q++) {
      fout[aos(g, x, g.ymin, bottom[q])] = fin[aos(g, x, g.ymin, opp_of(bottom[q]))];
      fout[aos(g, x, g.ymax, top[q])] = fin[aos(g, x, g.ymax, opp_of(top[q]))];
    }
  } else if (i < sx - 1 + sy - 1) {
    const int y = g.ymin + 1 + (i - (sx - 1));
#pragma unroll
    for (int q = 0; q < 3; q++) {
      fout[aos(g, g.xmin, y, left[q])] = fin[aos(g, g.xmin, y, opp_of(left[q]))];
      fout[aos(g, g.xmax, y, right[q])] = fin[aos(g, g.xmax, y, opp_of(right[q]))];
    }
  } else if (i == sx - 1 + sy - 1) {
    fout[aos(g, g.xmin, g.ymin, 7)] = fin[aos(g, g.xmin, g.ymin, 5)];
    fout[aos(g, g.xmin, g.ymax, 6)] = fin[aos(g, g.xmin, g.ymax, 8)];
    fout[aos(g, g.xmax, g.ymax, 5)] = fin[aos(g, g.xmax, g.ymax, 7)];
    fout[aos(g, g.xmax, g.ymin, 8)] = fin[aos(g, g.xmax, g.ymin, 6)];
  }
}

// pops driver :430-439
__global__ void k_ref_interior(GeomDev g, double *fout) {
  const int sx = g.xmax - g.xmin - 1, sy = g.ymax - g.ymin - 1;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (sx <= 0 || sy <= 0 || i >= sx * sy) return;
  const int x = g.xmin + 1 + i / sy, y = g.ymin + 1 + i % sy;
#pragma unroll
  for (int k = 0; k < 9; k++) fout[aos(g, x, y, k)] = w_of(k);
}

// force.cpp:8-144: per-node terms in parallel, then the four sides summed in
// node order by one thread.
__global__ void k_ref_force(GeomDev g, const double *f, double omega, double *out) {
  extern __shared__ double terms[];
  const int sx = g.xmax - g.xmin + 1, sy = g.ymax - g.ymin + 1;
  const int nterm = 2 * sy + 2 * sx;
  const double third = 1. / 3.;
  const double c = DSUB(1.0, DMUL(.5, omega));
  for (int i = threadIdx.x; i < nterm; i += blockDim.x) {
    int x, y, side;
    if (i < sy) { side = 0; x = g.xmin; y = g.ymin + i; }
    else if (i < 2 * sy) { side = 1; x = g.xmax; y = g.ymin + i - sy; }
    else if (i < 2 * sy + sx) { side = 2; y = g.ymax; x = g.xmin + i - 2 * sy; }
    else { side = 3; y = g.ymin; x = g.xmin + i - 2 * sy - sx; }
    double fn[9];
#pragma unroll
    for (int k = 0; k < 9; k++) fn[k] = f[aos(g, x, y, k)];
    double rho, pxx, pxy;
    pi_ref64(fn, rho, pxx, pxy);
    double v;
    if (side == 0) v = DADD(DMUL(rho, third), DMUL(c, pxx));
    else if (side == 1) v = DSUB(DMUL(-rho, third), DMUL(c, pxx));
    else if (side == 2) v = DMUL(-c, pxy);
    else v = DMUL(c, pxy);
    terms[i] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double side[4];
    const int len[4] = {sy, sy, sx, sx};
    int i = 0;
    for (int s = 0; s < 4; s++) {
      double v = terms[i];
      for (int q = 1; q < len[s]; q++) v = DADD(v, terms[i + q]);
      side[s] = v;
      i += len[s];
    }
    *out = DADD(DADD(DADD(side[0], side[1]), side[2]), side[3]);
  }
}

// generatePerturbedState.cpp:4-38 in two passes: fixed-order norm reduction,
// then the element-wise update.
__global__ void k_ref_perturb_norms(const double *fin, const double *snaps, int nsnap, int n,
                                    const double *pref, double *partials) {
  __shared__ double red[2][256 / 32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double n0 = 0.0, n1 = 0.0;
  if (i < n) {
    double mix = DMUL(pref[0], snaps[i]);
    for (int q = 1; q < nsnap; q++) mix = DADD(mix, DMUL(pref[q], snaps[(long long)q * n + i]));
    n0 = DMUL(fin[i], fin[i]);
    n1 = DMUL(mix, mix);
  }
  for (int o = 16; o > 0; o >>= 1) {
    n0 = DADD(n0, __shfl_down_sync(0xffffffffu, n0, o));
    n1 = DADD(n1, __shfl_down_sync(0xffffffffu, n1, o));
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = n0;
    red[1][threadIdx.x >> 5] = n1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a0 = red[0][0], a1 = red[1][0];
    for (int w = 1; w < 256 / 32; w++) {
      a0 = DADD(a0, red[0][w]);
      a1 = DADD(a1, red[1][w]);
    }
    partials[2 * blockIdx.x] = a0;
    partials[2 * blockIdx.x + 1] = a1;
  }
}

// The two norms summed over the blocks' partials in block order, once:
// out[0] = |f| / |mix| (the mix weight), out[1] = 1 / (1 + eps * sum(pref) * weight)
// (generatePerturbedState.cpp:22-36).
__global__ void k_ref_perturb_finalize(const double *pref, int nsnap, const double *partials,
                                       int nblocks, double eps, double *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double a0 = partials[0], a1 = partials[1];
  for (int b = 1; b < nblocks; b++) {
    a0 = DADD(a0, partials[2 * b]);
    a1 = DADD(a1, partials[2 * b + 1]);
  }
  const double weight = DDIV(__dsqrt_rn(a0), __dsqrt_rn(a1));
  double sum = pref[0];
  for (int q = 1; q < nsnap; q++) sum = DADD(sum, pref[q]);
  out[0] = weight;
  out[1] = DDIV(1., DADD(1.0, DMUL(DMUL(sum, eps), weight)));
}

// f <- (f + eps * mix * weight) / a with (weight, 1/a) from k_ref_perturb_finalize
__global__ void k_ref_perturb_apply(double *fin, const double *snaps, int nsnap, int n,
                                    const double *pref, const double *wa, double eps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double w = wa[0], inv = wa[1];
  double mix = DMUL(pref[0], snaps[i]);
  for (int q = 1; q < nsnap; q++) mix = DADD(mix, DMUL(pref[q], snaps[(long long)q * n + i]));
  fin[i] = DMUL(DADD(fin[i], DMUL(DMUL(eps, mix), w)), inv);
}

}  // namespace clbm

using namespace clbm;

extern "C" void clbm_set_error(const char *msg);
extern "C" int clbm_status_from_cuda(cudaError_t e);

static int check_geom(const clbm_geom *g) {
  if (!g || g->nx < 3 || g->ny < 3 || g->xmin < 0 || g->xmax >= g->nx || g->xmin > g->xmax ||
      g->ymin < 0 || g->ymax >= g->ny || g->ymin > g->ymax) {
    clbm_set_error("invalid geometry");
    return CLBM_ERR_INVALID;
  }
  return CLBM_OK;
}

static GeomDev to_dev(const clbm_geom *g) {
  return GeomDev{g->nx, g->ny, g->xmin, g->xmax, g->ymin, g->ymax};
}

extern "C" int clbm_ref_stream_collide(const clbm_geom *g, double *fin, double *fout, double *rho,
                                       double *ux, double *uy, double beta, double tau,
                                       void *stream) {
  if (int s = check_geom(g)) return s;
  if (!fin || !fout) return CLBM_ERR_INVALID;
  const int n = g->nx * g->ny;
  k_ref_stream_collide<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
      to_dev(g), fin, fout, rho, ux, uy, beta, nullptr, tau, 0.0);
  return clbm_status_from_cuda(cudaGetLastError());
}

extern "C" int clbm_ref_stream_collide_spatial(const clbm_geom *g, double *fin, double *fout,
                                               double *rho, double *ux, double *uy, double beta0,
                                               const double *map, double tau, double eps,
                                               void *stream) {
  if (int s = check_geom(g)) return s;
  if (!fin || !fout || !map) return CLBM_ERR_INVALID;
  const int n = g->nx * g->ny;
  k_ref_stream_collide<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
      to_dev(g), fin, fout, rho, ux, uy, beta0, map, tau, eps);
  return clbm_status_from_cuda(cudaGetLastError());
}

extern "C" int clbm_ref_walls_bb(const clbm_geom *g, double *fout, const double *fin,
                                 void *stream) {
  if (int s = check_geom(g)) return s;
  k_ref_walls<<<(g->nx + 127) / 128, 128, 0, (cudaStream_t)stream>>>(to_dev(g), fout, fin);
  return clbm_status_from_cuda(cudaGetLastError());
}

extern "C" int clbm_ref_square_bb(const clbm_geom *g, double *fout, const double *fin,
                                  void *stream) {
  if (int s = check_geom(g)) return s;
  const int nthreads = (g->xmax - g->xmin - 1) + (g->ymax - g->ymin - 1) + 1;
  k_ref_square<<<(nthreads + 127) / 128, 128, 0, (cudaStream_t)stream>>>(to_dev(g), fout, fin);
  return clbm_status_from_cuda(cudaGetLastError());
}

extern "C" int clbm_ref_interior_reset(const clbm_geom *g, double *fout, void *stream) {
  if (int s = check_geom(g)) return s;
  const int sx = g->xmax - g->xmin - 1, sy = g->ymax - g->ymin - 1;
  if (sx <= 0 || sy <= 0) return CLBM_OK;
  k_ref_interior<<<(sx * sy + 127) / 128, 128, 0, (cudaStream_t)stream>>>(to_dev(g), fout);
  return clbm_status_from_cuda(cudaGetLastError());
}

extern "C" int clbm_ref_force_on_square(const clbm_geom *g, const double *f, double omega,
                                        double *result, void *stream) {
  if (int s = check_geom(g)) return s;
  if (!f || !result) return CLBM_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  double *d_out = nullptr;
  cudaError_t e = cudaMallocAsync(&d_out, sizeof(double), st);
  if (e != cudaSuccess) return clbm_status_from_cuda(e);
  const int nterm = 2 * (g->xmax - g->xmin + 1) + 2 * (g->ymax - g->ymin + 1);
  k_ref_force<<<1, 256, nterm * sizeof(double), st>>>(to_dev(g), f, omega, d_out);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(result, d_out, sizeof(double), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(d_out, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return clbm_status_from_cuda(e);
}

extern "C" int clbm_ref_perturbed_state(double *fin, const double *snaps, double eps, int nsnap,
                                        int n, const double *prefactors, void *stream) {
  if (!fin || !snaps || !prefactors || nsnap < 1 || nsnap > 64 || n < 1) return CLBM_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  const int nb = (n + 255) / 256;
  double *d_buf = nullptr;
  cudaError_t e = cudaMallocAsync(&d_buf, sizeof(double) * (nsnap + 2 + 2 * (size_t)nb), st);
  if (e != cudaSuccess) return clbm_status_from_cuda(e);
  double *d_pref = d_buf, *d_wa = d_buf + nsnap, *d_part = d_buf + nsnap + 2;
  e = cudaMemcpyAsync(d_pref, prefactors, sizeof(double) * nsnap, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    k_ref_perturb_norms<<<nb, 256, 0, st>>>(fin, snaps, nsnap, n, d_pref, d_part);
    k_ref_perturb_finalize<<<1, 32, 0, st>>>(d_pref, nsnap, d_part, nb, eps, d_wa);
    k_ref_perturb_apply<<<nb, 256, 0, st>>>(fin, snaps, nsnap, n, d_pref, d_wa, eps);
    e = cudaGetLastError();
  }
  cudaFreeAsync(d_buf, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return clbm_status_from_cuda(e);
}

// ---------------------------------------------------------------------------
// clbm_ref_perturbed_state_noalloc: the same kernels as
// clbm_ref_perturbed_state, with their scratch (the snapshot prefactors and
// two norm partial sums per 256 values, the mix weight) in a fixed device
// array instead of a per-call allocation.  It serves callers that must not allocate device
// memory at all: code running under an allocator that already owns the whole
// device, or inside a time-critical loop where an allocation's implicit
// synchronisation is not acceptable.
namespace {
constexpr int NOALLOC_MAX_N = 1 << 20;                     // values per state, 9*Dx*Dy
constexpr int NOALLOC_MAX_BLOCKS = NOALLOC_MAX_N / 256;    // norm partials (pairs)
constexpr int NOALLOC_PREF = 64;                           // prefactor slots (nsnap <= 64)
// Shared by every call on a device and kept until the process exits
// (66 KB per device that loads the library): the prefactors, the mix weight
// and 1/a, then the norm partials.  Nothing in it has to start at zero: each
// call overwrites the prefactors, the weight pair and every partial it reads.
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_PREF + 2 + 2 * NOALLOC_MAX_BLOCKS];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
double *g_noalloc_addr[NOALLOC_MAX_DEVICES] = {};

// The array's device address on the current device, looked up once per
// device with that device current (the host-side symbol is not a device
// address and must never be passed to a kernel).
int noalloc_scratch(double **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return clbm_status_from_cuda(e);
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
    clbm_set_error("device ordinal beyond the no-alloc scratch table");
    return CLBM_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[dev]) {
    double *p = nullptr;
    e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
    if (e != cudaSuccess) return clbm_status_from_cuda(e);
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return CLBM_OK;
}
}  // namespace

extern "C" int clbm_ref_perturbed_state_noalloc(double *fin, const double *snaps, double eps,
                                                int nsnap, int n, const double *prefactors,
                                                void *stream) {
  if (!fin || !snaps || !prefactors || nsnap < 1 || nsnap > NOALLOC_PREF || n < 1) {
    clbm_set_error("invalid argument");
    return CLBM_ERR_INVALID;
  }
  if (n > NOALLOC_MAX_N) {
    clbm_set_error("n exceeds the no-alloc scratch limit of 1048576 values (9*Dx*Dy)");
    return CLBM_ERR_INVALID;
  }
  double *scratch = nullptr;
  if (int s = noalloc_scratch(&scratch)) return s;
  cudaStream_t st = (cudaStream_t)stream;
  const int nb = (n + 255) / 256;
  double *d_pref = scratch, *d_wa = scratch + NOALLOC_PREF, *d_part = scratch + NOALLOC_PREF + 2;
  cudaError_t e = cudaMemcpyAsync(d_pref, prefactors, sizeof(double) * nsnap,
                                  cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    k_ref_perturb_norms<<<nb, 256, 0, st>>>(fin, snaps, nsnap, n, d_pref, d_part);
    k_ref_perturb_finalize<<<1, 32, 0, st>>>(d_pref, nsnap, d_part, nb, eps, d_wa);
    k_ref_perturb_apply<<<nb, 256, 0, st>>>(fin, snaps, nsnap, n, d_pref, d_wa, eps);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return clbm_status_from_cuda(e);
}
