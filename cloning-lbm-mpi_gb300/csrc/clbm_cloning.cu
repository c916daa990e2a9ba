// clbm_cloning.cu -- device-side cloning step: the per-step drag on the square
// and the weight integral, then one CTA per run for the weights, the mean
// weight R_t, the copy numbers, the kill/duplicate correction, the copy table
// (labels) and the marks and random prefactors of new clones.  This replaces
// the master rank's gather/resample/broadcast of the reference
// (src/mpi_LBM_GK_pops_perturb.cpp:465-648).
#include <cstdint>

#include "clbm_internal.h"
#include "clbm_physics.cuh"

namespace clbm {

// ---------------------------------------------------------------------------
// Drag of every (clone, step): F_t = (West + East + North + South) * scale -
// shift, each side summed in the reference's node order (force.cpp:23-141,
// pops driver :445-449); one thread per (clone, step), clones fastest so the
// [term][clone] slabs are read coalesced.  Then one thread per clone forms
// s = dt * sum_t F_t in step order (:459, :465).
template <bool F64>
__global__ void k_drag_terms_sum(DevArrays d, int nruns, int total_clones) {
  using T = typename std::conditional<F64, double, float>::type;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = blockIdx.y;
  if (g >= total_clones) return;
  int r = 0;
  while (r + 1 < nruns && g >= d.runs[r + 1].clone_base) r++;
  const RunDev &R = d.runs[r];
  if (R.drag_mode != 0) return;  // momentum exchange: k_drag_me_sum
  const int c = g - R.clone_base;
  const int nc = R.nclones;
  const int sy = R.ymax - R.ymin + 1, sx = R.xmax - R.xmin + 1;
  const T *tt = (const T *)d.terms + (long long)t * d.term_slab + R.term_base + c;
  double side[4];
  int i = 0;
  const int len[4] = {sy, sy, sx, sx};
#pragma unroll
  for (int s = 0; s < 4; s++) {
    double v = (double)tt[(long long)i * nc];
    for (int q = 1; q < len[s]; q++) v = DADD(v, (double)tt[(long long)(i + q) * nc]);
    side[s] = v;
    i += len[s];
  }
  double F = DADD(DADD(DADD(side[0], side[1]), side[2]), side[3]);
  F = DMUL(F, R.force_scale);
  F = DSUB(F, R.force_shift);
  if (!isfinite(F)) atomicOr(d.err, (unsigned)ERR_NONFINITE_DRAG);
  d.drag[(long long)g * d.max_steps + t] = F;
}

// Momentum-exchange drag of every (clone, step) with a warp-shuffle
// reduction.  Block (32, 32) for 32 clones of one step: thread (tx, ty) adds
// the terms ty, ty + 32, ... of clone tx in FP64 (loads coalesced over the
// clones of the [term][clone] slab); the 32 x 32 partials are transposed
// through shared memory, so warp ty holds the partials of clone ty in its
// lanes, and an xor butterfly (offsets 16, 8, 4, 2, 1) completes the sum in a
// fixed order (the oracle restates the same order).
template <bool F64>
__global__ void __launch_bounds__(1024) k_drag_me_sum(DevArrays d, int nruns, int total_clones) {
  using T = typename std::conditional<F64, double, float>::type;
  __shared__ double part[32][33];
  const int tx = threadIdx.x, ty = threadIdx.y, t = blockIdx.y;
  const int g = blockIdx.x * 32 + tx;
  double v = 0.0;
  if (g < total_clones) {
    int r = 0;
    while (r + 1 < nruns && g >= d.runs[r + 1].clone_base) r++;
    const RunDev &R = d.runs[r];
    if (R.drag_mode == 1) {
      const int nc = R.nclones;
      const T *tt = (const T *)d.terms + (long long)t * d.term_slab + R.term_base + (g - R.clone_base);
      for (int i = ty; i < R.nterms; i += 32) v = DADD(v, (double)tt[(long long)i * nc]);
    }
  }
  part[ty][tx] = v;
  __syncthreads();
  double w = part[tx][ty];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) w = DADD(w, __shfl_xor_sync(0xffffffffu, w, o));
  const int gc = blockIdx.x * 32 + ty;
  if (tx != 0 || gc >= total_clones) return;
  int r = 0;
  while (r + 1 < nruns && gc >= d.runs[r + 1].clone_base) r++;
  const RunDev &R = d.runs[r];
  if (R.drag_mode != 1) return;
  const double F = DSUB(DMUL(w, R.force_scale), R.force_shift);
  if (!isfinite(F)) atomicOr(d.err, (unsigned)ERR_NONFINITE_DRAG);
  d.drag[(long long)gc * d.max_steps + t] = F;
}

__global__ void k_drag_integrate(DevArrays d, int nruns, int total_clones, int steps) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total_clones) return;
  int r = 0;
  while (r + 1 < nruns && g >= d.runs[r + 1].clone_base) r++;
  const double *drag = d.drag + (long long)g * d.max_steps;
  double acc = drag[0];
  for (int t = 1; t < steps; t++) acc = DADD(acc, drag[t]);
  d.sacc[g] = DMUL(acc, d.runs[r].dt);
}

cudaError_t launch_drag_reduce(bool f64, const DevArrays &d, int nruns, int total_clones,
                               int steps, bool stress, bool momentum, cudaStream_t s) {
  if (stress) {
    dim3 grid((total_clones + 127) / 128, steps);
    if (f64)
      k_drag_terms_sum<true><<<grid, 128, 0, s>>>(d, nruns, total_clones);
    else
      k_drag_terms_sum<false><<<grid, 128, 0, s>>>(d, nruns, total_clones);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (momentum) {
    dim3 grid((total_clones + 31) / 32, steps), block(32, 32);
    if (f64)
      k_drag_me_sum<true><<<grid, block, 0, s>>>(d, nruns, total_clones);
    else
      k_drag_me_sum<false><<<grid, block, 0, s>>>(d, nruns, total_clones);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  k_drag_integrate<<<(total_clones + 127) / 128, 128, 0, s>>>(d, nruns, total_clones, steps);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Block-wide scans over n items, each thread owning a contiguous chunk.
constexpr int CLONE_THREADS = 1024;

template <typename V>
__device__ V block_exclusive_scan_total(V v, V *sh, V &total) {
  // v: this thread's chunk sum; returns the exclusive prefix of the chunk sums
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  V x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    V y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x = x + y;
  }
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  if (warp == 0) {
    V w = lane < (CLONE_THREADS / 32) ? sh[lane] : V(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      V y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w = w + y;
    }
    sh[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  const V before = warp > 0 ? sh[warp - 1] : V(0);
  total = sh[CLONE_THREADS / 32 - 1];
  const V excl = before + x - v;
  __syncthreads();
  return excl;
}

// One CTA per run.
__global__ void __launch_bounds__(CLONE_THREADS) k_clone(DevArrays d, int nruns) {
  __shared__ int shi[32];
  __shared__ double shd[32];
  __shared__ double sh_rbar, sh_logr, sh_u, sh_max;
  __shared__ int sh_status;
  const int r = blockIdx.x;
  const RunDev &R = d.runs[r];
  RunState &st = d.state[r];
  const int nc = R.nclones;
  const int g0 = R.clone_base;
  const int per = (nc + CLONE_THREADS - 1) / CLONE_THREADS;
  const int j0 = min(nc, threadIdx.x * per), j1 = min(nc, j0 + per);
  int *ncop = d.scratch_i + 4LL * g0 + 4LL * r;  // nc copy numbers
  int *temp = ncop + nc;                         // 2nc+2 sampling array
  int *extras = temp + 2 * nc + 2;               // nc surplus copies' parents
  double *pre = d.scratch_d + g0;                // nc prefix sums
  const bool systematic = R.resample_mode == 1;
  if (threadIdx.x == 0) {
    sh_status = 0;
    sh_rbar = NAN;
    sh_logr = NAN;
  }

  // ---- weights (pops driver :465-469) ----
  double locmax = -INFINITY;
  for (int j = j0; j < j1; j++) {
    const double lw = DMUL(R.alpha, d.sacc[g0 + j]);
    const double s = exp(lw);
    d.weights[g0 + j] = s;
    locmax = fmax(locmax, lw);
  }
  __syncthreads();

  int drawn_local = 0;
  if (!systematic) {
    // ---- mean weight R_t: per-rank sequential sums, rank 0 first (:487-512)
    if (threadIdx.x == 0) {
      const int local = nc / R.ranks;
      double total = 0.0;
      for (int q = 0; q < R.ranks; q++) {
        double part = d.weights[g0 + q * local];
        for (int j = q * local + 1; j < (q + 1) * local; j++) part = DADD(part, d.weights[g0 + j]);
        total = q == 0 ? part : DADD(total, part);
      }
      const double rbar = DDIV(total, (double)nc);
      sh_rbar = rbar;
      sh_logr = log(rbar);
      if (!isfinite(rbar) || !(rbar > 0.0)) sh_status = ERR_WEIGHT_OVERFLOW;
    }
    __syncthreads();
    if (sh_status) goto fail;
    // ---- copy numbers n_j = floor(s_j/R + drand48()) on rank 0's stream (:514-520)
    const uint64_t x0 = st.d48[0];
    for (int j = j0; j < j1; j++) {
      const double a = d48_value(d48_skip(x0, (uint64_t)j + 1));
      const double v = floor(DADD(DDIV(d.weights[g0 + j], sh_rbar), a));
      int n = 0;
      if (!(v >= 0.0 && v <= 2.0 * nc + 1.0))
        atomicOr(&sh_status, (int)ERR_WEIGHT_OVERFLOW);
      else
        n = (int)v;
      ncop[j] = n;
      d.copies_pre[g0 + j] = n;
      drawn_local += n;
    }
  } else {
    // ---- systematic: log-domain weights, one Philox uniform per interval
    for (int o = 16; o > 0; o >>= 1) locmax = fmax(locmax, __shfl_xor_sync(0xffffffffu, locmax, o));
    if ((threadIdx.x & 31) == 0) shd[threadIdx.x >> 5] = locmax;
    __syncthreads();
    if (threadIdx.x == 0) {
      double m = shd[0];
      for (int i = 1; i < CLONE_THREADS / 32; i++) m = fmax(m, shd[i]);
      sh_max = m;
      sh_u = philox_uniform(R.seed, (uint32_t)st.interval, 0, 0, (R.run_id << 4) | DOM_SYSTEMATIC);
      if (!isfinite(m)) sh_status = ERR_WEIGHT_OVERFLOW;
    }
    __syncthreads();
    if (sh_status) goto fail;
    double acc = 0.0;
    for (int j = j0; j < j1; j++) {
      acc = DADD(acc, exp(DSUB(DMUL(R.alpha, d.sacc[g0 + j]), sh_max)));
      pre[j] = acc;
    }
    double tot;
    const double off = block_exclusive_scan_total<double>(acc, shd, tot);
    for (int j = j0; j < j1; j++) pre[j] = DADD(pre[j], off);
    if (threadIdx.x == 0) {
      sh_logr = DADD(sh_max, log(DDIV(tot, (double)nc)));
      sh_rbar = exp(sh_logr);
    }
    __syncthreads();
    const double last = pre[nc - 1];
    for (int j = j0; j < j1; j++) {
      const double cj = DMUL(DDIV(pre[j], last), (double)nc);
      const double cprev = j == 0 ? 0.0 : DMUL(DDIV(pre[j - 1], last), (double)nc);
      const int n = (int)(floor(DADD(cj, sh_u)) - floor(DADD(cprev, sh_u)));
      ncop[j] = n;
      d.copies_pre[g0 + j] = n;
      drawn_local += n;
    }
  }
  __syncthreads();
  if (sh_status) goto fail;
  {
    // ---- sampling array temp[]: j repeated n_j times (:524-532)
    int drawn;
    const int off = block_exclusive_scan_total<int>(drawn_local, shi, drawn);
    if (drawn > 2 * nc + 2) {
      if (threadIdx.x == 0) sh_status = ERR_RESAMPLE;
    } else {
      int o = off;
      for (int j = j0; j < j1; j++)
        for (int i = 0; i < ncop[j]; i++) temp[o++] = j;
    }
    __syncthreads();
    if (sh_status) goto fail;
    // ---- kill / duplicate correction with glibc rand() (:540-571)
    if (threadIdx.x == 0) {
      const int delta = drawn - nc;
      GlibcRand rnd = st.rnd;
      if (delta > 0) {
        for (int i = 0; i < delta; i++) {
          const int idx = glibc_rand_next(rnd) % (drawn - i);
          const int victim = temp[idx];
          temp[idx] = temp[drawn - i - 1];
          ncop[victim]--;
        }
      } else if (delta < 0) {
        if (drawn == 0) {
          sh_status = ERR_RESAMPLE;
        } else {
          for (int i = 0; i < -delta; i++) ncop[temp[glibc_rand_next(rnd) % drawn]]++;
        }
      }
      st.rnd = rnd;
      st.ncopies_drawn = drawn;
      if (!systematic) st.d48[0] = d48_skip(st.d48[0], (uint64_t)nc);
    }
    __syncthreads();
    if (sh_status) goto fail;
    // ---- copy table: the m-th surplus copy (ascending parent) fills the m-th
    // lowest killed slot (:590-619)
    int killed_local = 0, extra_local = 0;
    for (int j = j0; j < j1; j++) {
      const int n = ncop[j];
      d.copies_post[g0 + j] = n;
      killed_local += n == 0;
      extra_local += n > 1 ? n - 1 : 0;
    }
    int killed, extra;
    const int koff = block_exclusive_scan_total<int>(killed_local, shi, killed);
    const int eoff = block_exclusive_scan_total<int>(extra_local, shi, extra);
    if (killed != extra) {
      if (threadIdx.x == 0) sh_status = ERR_RESAMPLE;
    } else {
      int o = eoff;
      for (int j = j0; j < j1; j++)
        for (int i = 1; i < ncop[j]; i++) extras[o++] = j;
    }
    __syncthreads();
    if (sh_status) goto fail;
    int k = koff;
    for (int j = j0; j < j1; j++) {
      const bool dead = ncop[j] == 0;
      d.labels[g0 + j] = dead ? extras[k] : j;
      d.mark[g0 + j] = dead ? 1 : 0;
      k += dead;
    }
    // ---- snapshot-mix prefactors of the new clones: rank q's stream, 'nsnap'
    // draws per marked clone in slot order (generatePerturbedState.cpp:15,
    // drawn at the start of the next interval, :412-416)
    if (R.perturb_mode == 1) {
      // mrank[j] = marked slots before j (exclusive scan of the marks in slot
      // order, in the sampling array's space, which is free again); a marked
      // slot j of rank q is the (mrank[j] - mrank[q*local])-th marked slot of
      // q's block and takes that many nsnap-blocks further into q's stream
      const int local = nc / R.ranks;
      // (the marked slots are the killed ones: koff is that scan already)
      int *mrank = temp;
      {
        int o = koff;
        for (int j = j0; j < j1; j++) {
          mrank[j] = o;
          o += ncop[j] == 0;
        }
        if (threadIdx.x == 0) mrank[nc] = killed;
      }
      __syncthreads();
      for (int j = j0; j < j1; j++) {
        if (ncop[j] != 0) continue;
        const int q = j / local;
        const int m = mrank[j] - mrank[q * local];
        const uint64_t x = st.d48[q];
        double *p = d.prefactors + (long long)(g0 + j) * MAX_SNAP;
        for (int s = 0; s < R.nsnap; s++)
          p[s] = d48_value(d48_skip(x, (uint64_t)m * R.nsnap + s + 1));
      }
      __syncthreads();
      if (threadIdx.x < R.ranks) {
        const int q = threadIdx.x;
        const int cnt = mrank[(q + 1) * local] - mrank[q * local];
        st.d48[q] = d48_skip(st.d48[q], (uint64_t)cnt * R.nsnap);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      st.ncomm = killed;
      st.rbar = sh_rbar;
      st.logr = sh_logr;
      if (st.interval < d.max_intervals) {
        d.rvalues[(long long)r * d.max_intervals + st.interval] = sh_rbar;
        d.logr[(long long)r * d.max_intervals + st.interval] = sh_logr;
      }
      st.interval += 1;
    }
    return;
  }
fail:
  __syncthreads();
  // leave every slot on itself and flag the error; the host reports it
  for (int j = j0; j < j1; j++) {
    d.labels[g0 + j] = j;
    d.mark[g0 + j] = 0;
  }
  if (threadIdx.x == 0) {
    atomicOr(d.err, (unsigned)sh_status);
    st.rbar = sh_rbar;
    st.logr = sh_logr;
    st.interval += 1;
  }
}

// SCGF estimator in FP64 (post_processing/read_rvalue.py:14-20 restated
// with its hard-coded dT replaced by the run's): psi = sum_t log R_t /
// (count * dT) over intervals [first, first+count), summed in order.
__global__ void k_scgf(const double *logr, int first, int count, double dT, double *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double acc = logr[first];
  for (int t = 1; t < count; t++) acc = DADD(acc, logr[first + t]);
  out[0] = DDIV(acc, DMUL((double)count, dT));
}

cudaError_t launch_scgf(const double *logr, int first, int count, double dT, double *out,
                        cudaStream_t s) {
  k_scgf<<<1, 32, 0, s>>>(logr, first, count, dT, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// History for lineage reconstruction: every interval's drag series and the
// labels of the clone step that ends it, indexed by the device-side interval
// counter so that graph replays record correctly.
__global__ void k_hist_drag(DevArrays d, int total_clones, int steps, double *hist, int max_hist) {
  const int t = d.state[0].interval;  // interval being finished (before its clone step)
  if (t >= max_hist) return;
  const long long n = (long long)total_clones * d.max_steps;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    hist[(long long)t * n + i] = d.drag[i];
}

__global__ void k_hist_labels(DevArrays d, int total_clones, int *hist, int max_hist) {
  const int t = d.state[0].interval - 1;  // clone step just completed
  if (t < 0 || t >= max_hist) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total_clones; i += gridDim.x * blockDim.x)
    hist[(long long)t * total_clones + i] = d.labels[i];
}

cudaError_t launch_hist_drag(const DevArrays &d, int total_clones, int steps, double *hist, int max_hist,
                             cudaStream_t s) {
  k_hist_drag<<<592, 256, 0, s>>>(d, total_clones, steps, hist, max_hist);
  return cudaGetLastError();
}

cudaError_t launch_hist_labels(const DevArrays &d, int total_clones, int *hist, int max_hist,
                               cudaStream_t s) {
  k_hist_labels<<<(total_clones + 255) / 256, 256, 0, s>>>(d, total_clones, hist, max_hist);
  return cudaGetLastError();
}

// Ancestors of the final slots (post_processing/reconstruction.cpp:72-108
// restated): slot_{n-1} = j, slot_t = labels_t[slot_{t+1}].
__global__ void k_ancestors(const int *hist_labels, int total_clones, int clone_base, int nclones,
                            int n, int *anc) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nclones) return;
  int slot = j;
  anc[(long long)j * n + (n - 1)] = slot;
  for (int t = n - 2; t >= 0; t--) {
    slot = hist_labels[(long long)t * total_clones + clone_base + slot];
    anc[(long long)j * n + t] = slot;
  }
}

// out[j][t*steps + s] = drag of slot anc[j][t] in interval t, step s
__global__ void k_gather_lineages(const double *hist_drag, const int *anc, int total_clones,
                                  int clone_base, int nclones, int n, int steps, int max_steps,
                                  double *out) {
  const long long total = (long long)nclones * n * steps;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int s = (int)(i % steps);
    const long long q = i / steps;
    const int t = (int)(q % n), j = (int)(q / n);
    const int slot = anc[(long long)j * n + t];
    out[i] = hist_drag[((long long)t * total_clones + clone_base + slot) * max_steps + s];
  }
}

cudaError_t launch_reconstruct(const double *hist_drag, const int *hist_labels, int total_clones,
                               int clone_base, int nclones, int n, int steps, int max_steps,
                               int *anc, double *out, cudaStream_t s) {
  k_ancestors<<<(nclones + 127) / 128, 128, 0, s>>>(hist_labels, total_clones, clone_base, nclones, n, anc);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_gather_lineages<<<1184, 256, 0, s>>>(hist_drag, anc, total_clones, clone_base, nclones, n, steps,
                                         max_steps, out);
  return cudaGetLastError();
}

cudaError_t launch_clone(const DevArrays &d, int nruns, cudaStream_t s) {
  k_clone<<<nruns, CLONE_THREADS, 0, s>>>(d, nruns);
  return cudaGetLastError();
}

}  // namespace clbm
