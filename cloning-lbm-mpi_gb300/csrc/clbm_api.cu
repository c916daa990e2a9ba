// clbm_api.cu -- the sampler context and the C ABI declared in include/clbm.h.
//
// A context owns every clone of one or several independent runs in two
// structure-of-arrays population buffers (ping-pong), the drag-term slabs of
// one interval, and the per-clone arrays of the cloning step.  Between
// intervals buffer `s_buf` holds the pre-collision state S of every slot; the
// pending labels/marks say which parent each slot copies and which slots are
// perturbed when the next interval starts.
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <string>
#include <algorithm>
#include <vector>

#include "../../include/clbm.h"
#include "clbm_internal.h"

using namespace clbm;

static thread_local std::string g_last_error;

extern "C" void clbm_set_error(const char *msg) { g_last_error = msg ? msg : ""; }

extern "C" int clbm_status_from_cuda(cudaError_t e) {
  if (e == cudaSuccess) return CLBM_OK;
  g_last_error = std::string("CUDA: ") + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? CLBM_ERR_NOMEM : CLBM_ERR_CUDA;
}

#define CK(call)                                      \
  do {                                                \
    cudaError_t _e = (call);                          \
    if (_e != cudaSuccess) return clbm_status_from_cuda(_e); \
  } while (0)

static int fail(int status, const char *msg) {
  g_last_error = msg;
  return status;
}

struct GraphEntry {
  cudaGraphExec_t exec = nullptr;
  int sbuf = -1, steps = -1;
};

struct clbm_ctx {
  int nruns = 0, precision = 0, max_steps = 0, flags = 0;
  std::vector<clbm_run_desc> desc;
  std::vector<RunDev> runs_h;
  int total_clones = 0, total_blocks = 0;
  size_t pop_elems = 0, elem_size = 8;
  void *pop[2] = {nullptr, nullptr};
  int s_buf = 0;
  int last_steps = 0;
  bool any_mix = false;
  bool any_stress = false, any_momentum = false;  // drag modes present
  DevArrays d{};
  cudaStream_t stream = nullptr;
  GraphEntry graphs[4];
  int *d_identity = nullptr;  // 0..Nc-1 of every run, to reset pending labels
  std::vector<char> snaps_loaded;
  // optional timing of the step kernels: one event pair around the T step
  // launches of every eagerly enqueued interval
  bool profiling = false;
  std::vector<cudaEvent_t> ev;  // 2 per profiled interval
  int ev_used = 0;
  int prof_steps = 0;
  std::vector<cudaEvent_t> fev;  // 2 per profiled interval with random fields
  int fev_used = 0;
  int max_nodes = 0;
  int total_tiles[3] = {0, 0, 0};
  int step_variant = 0;  // FP32 step launch variant (clbm_autotune)
  // interval kernel of each run (FP32): cluster size of the cluster-resident
  // kernel, 0 = the streaming step kernel, and its thread variant.  The
  // streaming runs share one step launch per step; every cluster-resident run
  // is one launch per interval on its own side stream, concurrent with them.
  std::vector<int> run_cs, run_tv;
  // band split of each cluster-resident run (row0[0..cs]; empty = even)
  std::vector<std::vector<int>> run_rows;
  bool stream_subset = false;       // some runs are cluster-resident: step the rest through...
  RunDev *d_runs_stream = nullptr;  // ...this table (their descriptors, own tile bases)
  std::vector<RunDev> stream_h;
  int stream_nruns = 0, stream_tiles[3] = {0, 0, 0};
  std::vector<cudaStream_t> side;   // side stream i carries the i-th cluster-resident run
  std::vector<cudaEvent_t> fork_join;  // [0] fork, [1 + i] side stream i done
  bool pending = false;  // a clone step's copies/perturbations await the next interval
  // pinned staging of clbm_run_sampler_outputs: two slots, each the drag
  // series (total_clones x max_steps), labels and weights of one interval
  double *h_drag[2] = {nullptr, nullptr}, *h_weights[2] = {nullptr, nullptr};
  int *h_labels[2] = {nullptr, nullptr};
  cudaEvent_t h_ready[2] = {nullptr, nullptr};
  // random body-force fields (forcing variant)
  bool any_field = false;
  float *d_spec = nullptr, *d_maps = nullptr;
  float2 *d_tw = nullptr, *d_ybuf = nullptr;
  float *d_fa = nullptr;  // stage-1 DFT operand images of the field runs
  int *d_flist = nullptr; // kept embedding rows and columns of the field runs
  int field_max_w = 0, field_max_m1 = 0, field_max_m2 = 0, field_max_tiles2 = 0;
  std::vector<int> field_negative;  // spectrum entries below -1e-15 (clamped to 0)
  // lineage history (clbm_enable_history)
  double *hist_drag = nullptr;
  int *hist_labels = nullptr;
  int hist_max = 0, hist_steps = 0;
  bool hist_steps_varied = false;
  int *d_zeros = nullptr;
  // adjoint: forward checkpoints of P every adj_every steps
  struct {
    int steps = 0, every = 0;
    char *s0 = nullptr, *ckpt = nullptr, *seg = nullptr, *sig[2] = {nullptr, nullptr};
    size_t nckpt = 0, nseg = 0;
    int result = -1;  // which sig buffer holds sigma_0 after the backward
  } adj;
};

extern "C" const char *clbm_strerror(int status) {
  switch (status) {
    case CLBM_OK: return "ok";
    case CLBM_ERR_INVALID: return "invalid argument or call order";
    case CLBM_ERR_CUDA: return "CUDA runtime error";
    case CLBM_ERR_DEVICE: return "device error word set";
    case CLBM_ERR_NOMEM: return "out of memory";
    case CLBM_ERR_IO: return "I/O error";
    default: return "unknown status";
  }
}

extern "C" const char *clbm_last_error(void) { return g_last_error.c_str(); }
extern "C" int clbm_version(void) { return 10000; }
extern "C" int clbm_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

static bool geometry_ok(const clbm_run_desc &r) {
  if (r.width < 3 || r.height < 3 || r.nclones < 1) return false;
  if (r.xmin < 0 || r.xmax >= r.width || r.xmin > r.xmax) return false;
  if (r.ymin < 1 || r.ymax > r.height - 2 || r.ymin > r.ymax) return false;
  const unsigned long long nodes = (unsigned long long)r.width * r.height;
  if ((nodes - 1) * (unsigned long long)(r.width - 1) >= (1ULL << 32)) return false;
  return true;
}

// FP32 collision constants with exactly consistent relaxation factors:
// c2 = omega/12 rounded to a multiple of 2^-25, c13 = (omega - 4 c2)/2
// rounded to a multiple of 2^-24, omega' = 2 c13 + 4 c2 (a multiple of 2^-23,
// within 3e-8 of omega), om1 = 1 - omega' and cforce = 1 - omega'/2; every
// one of them is exactly representable in FP32, which is checked.
static bool f32_collision_constants(double omega, RunDev &R) {
  const double c2 = std::nearbyint(omega / 12.0 * 33554432.0) / 33554432.0;
  const double c13 = std::nearbyint((omega - 4.0 * c2) / 2.0 * 16777216.0) / 16777216.0;
  const double om = 2.0 * c13 + 4.0 * c2;
  if (!(c2 > 0.0 && c13 > 0.0 && om > 0.0 && om <= 2.0)) return false;
  R.f_omega = (float)om;
  R.f_om1 = (float)(1.0 - om);
  R.f_c13 = (float)c13;
  R.f_c2 = (float)c2;
  R.f_cforce = (float)(1.0 - 0.5 * om);
  return (double)R.f_omega == om && (double)R.f_om1 == 1.0 - om && (double)R.f_c13 == c13 &&
         (double)R.f_c2 == c2 && (double)R.f_cforce == 1.0 - 0.5 * om;
}

static void destroy_graphs(clbm_ctx *c) {
  for (auto &g : c->graphs) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = GraphEntry{};
  }
}

extern "C" int clbm_destroy(clbm_ctx *c) {
  if (!c) return CLBM_OK;
  destroy_graphs(c);
  for (cudaStream_t t : c->side) cudaStreamDestroy(t);
  for (cudaEvent_t e : c->fork_join) cudaEventDestroy(e);
  void *bufs[] = {c->d_runs_stream, c->pop[0], c->pop[1], c->d.runs, c->d.state, c->d.sacc, c->d.drag, c->d.weights,
                  c->d.labels, c->d.mark, c->d.copies_pre, c->d.copies_post, c->d.prefactors,
                  c->d.pert, c->d.partials, c->d.scratch_i, c->d.scratch_d, c->d.snaps,
                  c->d.rvalues, c->d.logr, c->d.err, c->d.terms, c->d_identity, c->d_zeros,
                  c->adj.s0, c->adj.ckpt, c->adj.seg, c->adj.sig[0], c->adj.sig[1],
                  c->hist_drag, c->hist_labels, c->d_spec, c->d_maps, c->d_tw, c->d_ybuf, c->d_fa, c->d_flist};
  for (void *b : bufs)
    if (b) cudaFree(b);
  for (cudaEvent_t e : c->ev) cudaEventDestroy(e);
  for (cudaEvent_t e : c->fev) cudaEventDestroy(e);
  for (int k = 0; k < 2; k++) {
    void *hb[] = {c->h_drag[k], c->h_weights[k], c->h_labels[k]};
    for (void *b : hb)
      if (b) cudaFreeHost(b);
    if (c->h_ready[k]) cudaEventDestroy(c->h_ready[k]);
  }
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return CLBM_OK;
}

template <typename T>
static cudaError_t dalloc(T *&p, size_t n) {
  if (n == 0) n = 1;
  return cudaMalloc((void **)&p, n * sizeof(T));
}

extern "C" int clbm_create(const clbm_run_desc *runs, int nruns, int precision, int max_steps,
                           int flags, clbm_ctx **out) {
  if (!out) return fail(CLBM_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (!runs || nruns < 1 || nruns > 1024) return fail(CLBM_ERR_INVALID, "nruns out of range");
  if (precision != CLBM_FP64 && precision != CLBM_FP32)
    return fail(CLBM_ERR_INVALID, "unknown precision");
  if (max_steps < 1 || max_steps > 65535) return fail(CLBM_ERR_INVALID, "max_steps outside [1, 65535]");
  for (int r = 0; r < nruns; r++) {
    const clbm_run_desc &d = runs[r];
    if (!geometry_ok(d)) return fail(CLBM_ERR_INVALID, "invalid run geometry");
    const int ranks = d.ranks < 1 ? 1 : d.ranks;
    if (ranks > MAX_RANKS || d.nclones % ranks) return fail(CLBM_ERR_INVALID, "ranks must divide nclones (<= 64)");
    if (d.perturb_mode < 0 || d.perturb_mode > 2) return fail(CLBM_ERR_INVALID, "unknown perturb_mode");
    if (d.resample_mode < 0 || d.resample_mode > 1) return fail(CLBM_ERR_INVALID, "unknown resample_mode");
    if (d.drag_mode != CLBM_DRAG_STRESS && d.drag_mode != CLBM_DRAG_MOMENTUM)
      return fail(CLBM_ERR_INVALID, "unknown drag_mode");
    if (d.drag_mode == CLBM_DRAG_MOMENTUM && (d.xmax - d.xmin < 2 || d.ymax - d.ymin < 2))
      return fail(CLBM_ERR_INVALID, "momentum-exchange drag needs a square with interior nodes (side >= 3)");
    if (d.perturb_mode == CLBM_PERTURB_MIX && (d.nsnap < 1 || d.nsnap > MAX_SNAP))
      return fail(CLBM_ERR_INVALID, "snapshot mix needs 1 <= nsnap <= 64");
    if (!(d.tau > 0.5)) return fail(CLBM_ERR_INVALID, "tau must exceed 1/2");
    if (d.field_mode < 0 || d.field_mode > 1) return fail(CLBM_ERR_INVALID, "unknown field_mode");
    if (d.field_mode && (d.width > 1024 || d.height > 1024 || d.field_steps < 0))
      return fail(CLBM_ERR_INVALID, "random field needs W, H <= 1024 and field_steps >= 0");
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return fail(CLBM_ERR_CUDA, "no CUDA device");
  }
  clbm_ctx *c = new clbm_ctx();
  c->nruns = nruns;
  c->precision = precision;
  c->max_steps = max_steps;
  c->flags = flags;
  c->elem_size = precision == CLBM_FP64 ? 8 : 4;
  c->desc.assign(runs, runs + nruns);
  c->snaps_loaded.assign(nruns, 0);
  c->runs_h.resize(nruns);
  long long pop = 0, terms = 0, snaps = 0, spec = 0, tw = 0, ybuf = 0, maps = 0, fa = 0, flist = 0;
  std::vector<float> h_fa;
  std::vector<int> h_flist;
  std::vector<float> h_spec;
  std::vector<float2> h_tw;
  c->field_negative.assign(nruns, 0);
  int clones = 0, blocks = 0;
  for (int r = 0; r < nruns; r++) {
    const clbm_run_desc &d = runs[r];
    RunDev &R = c->runs_h[r];
    memset(&R, 0, sizeof(R));
    R.W = d.width;
    R.H = d.height;
    R.xmin = d.xmin;
    R.xmax = d.xmax;
    R.ymin = d.ymin;
    R.ymax = d.ymax;
    R.nclones = d.nclones;
    R.clone_base = clones;
    R.block_base = blocks;
    R.nodes = d.width * d.height;
    R.blocks_per_clone = (R.nodes + STEP_BLOCK - 1) / STEP_BLOCK;
    R.nterms = 2 * (d.ymax - d.ymin + 1) + 2 * (d.xmax - d.xmin + 1);
    R.div_w = (unsigned)(((1ULL << 32) + (unsigned long long)d.width - 1) / (unsigned long long)d.width);
    R.plane = ((long long)R.nodes + 63) / 64 * 64;
    for (int q = 0; q < 3; q++) {
      const int tb = 128 << q;
      R.tiles[q] = (R.nodes + tb - 1) / tb;
      // clone = umulhi(local tile, ceil(2^32/tiles)) is exact while
      // local * (tiles - 1) < 2^32
      if ((unsigned long long)d.nclones * R.tiles[q] * (unsigned long long)(R.tiles[q] - 1) >= (1ULL << 32)) {
        delete c;
        return fail(CLBM_ERR_INVALID, "too many clones for the lattice size in one run (clones * tiles^2 >= 2^32)");
      }
      R.tiles_div[q] = (unsigned)(((1ULL << 32) + R.tiles[q] - 1) / R.tiles[q]);
      R.tile_base[q] = c->total_tiles[q];
      c->total_tiles[q] += d.nclones * R.tiles[q];
    }
    R.pop_base = pop;
    R.term_base = terms;
    R.snap_base = snaps;
    // the reference's scalar set-up (streamCollCompute.cpp:11-12)
    R.tau = d.tau;
    R.omega = 1. / d.tau;
    R.om1 = 1.0 - R.omega;
    R.cforce = 1.0 - 0.5 * R.omega;
    R.beta = d.beta;
    for (int k = 0; k < 9; k++) R.wcb[k] = w_of(k) * R.cforce * d.beta;
    R.alpha = d.alpha;
    R.force_scale = d.force_scale;
    R.force_shift = d.force_shift;
    R.dt = d.dt;
    R.eps = d.eps;
    if (!f32_collision_constants(R.omega, R)) {
      delete c;
      return fail(CLBM_ERR_INVALID, "tau out of range for the FP32 collision (need 0.5 < tau)");
    }
    R.f_beta = (float)d.beta;
    R.f_force = f32_force(R.f_beta, R.f_cforce);
    R.f_pairs = f32_pairs(R.f_omega, R.f_om1, R.f_c13, R.f_c2, R.f_force);
    R.perturb_mode = d.perturb_mode;
    R.resample_mode = d.resample_mode;
    R.drag_mode = d.drag_mode;
    (d.drag_mode == CLBM_DRAG_MOMENTUM ? c->any_momentum : c->any_stress) = true;
    R.ranks = d.ranks < 1 ? 1 : d.ranks;
    R.nsnap = d.perturb_mode == CLBM_PERTURB_MIX ? d.nsnap : 0;
    R.seed = d.seed;
    R.run_id = (unsigned)r;
    if (d.field_mode) {
      // circulant embedding of exp(-r^2/(2 sigma^2)) on (2W-1) x (2H-1): the
      // spectrum is separable, lambda[a][b] = l1[a] l2[b] / (M1 M2), l = DFT
      // of the 1-D embedded Gaussian g[j] = exp(-min(j, M-j)^2 / (2 sigma^2))
      const double sig = d.field_sigma > 0 ? d.field_sigma : 32.0;
      const int M1 = 2 * d.width - 1, M2 = 2 * d.height - 1;
      auto spectrum = [&](int M) {
        std::vector<double> g(M), l(M), cs(M);
        for (int j = 0; j < M; j++) {
          const double dd = std::min(j, M - j);
          g[j] = std::exp(-dd * dd / (2 * sig * sig));
          cs[j] = std::cos(2.0 * M_PI * j / M);
        }
        for (int a = 0; a < M; a++) {
          double acc = 0.0;
          for (int j = 0; j < M; j++) acc += g[j] * cs[(int)(((long long)a * j) % M)];
          l[a] = acc;
        }
        return l;
      };
      const std::vector<double> l1 = spectrum(M1), l2 = spectrum(M2);
      // The modes kept.  lambda[a][b] = l1[a] l2[b] / (M1 M2), so a row a whose
      // |l1[a]| is below 1e-16 of the largest has every amplitude sqrt(lambda)
      // below 1e-8 of the largest, and likewise a column b.  Left out, all such
      // modes together (at most M1 M2 of them, independent normals) change the
      // field by under 3e-6 of its RMS -- far below the TF32 rounding of the
      // transform.  A smooth field (sigma of the order of the lattice) keeps a
      // few percent of the rows and columns; a rough one keeps them all.
      auto kept = [](const std::vector<double> &l) {
        double mx = 0.0;
        for (double v : l) mx = std::max(mx, std::fabs(v));
        std::vector<int> idx;
        for (int i = 0; i < (int)l.size(); i++)
          if (std::fabs(l[i]) > 1e-16 * mx) idx.push_back(i);
        return idx;
      };
      const std::vector<int> alist = kept(l1), blist = kept(l2);
      const int na = (int)alist.size(), nb = (int)blist.size();
      R.field_mode = 1;
      R.field_steps = d.field_steps;
      R.M1 = M1;
      R.M2 = M2;
      R.field_eps = d.field_eps;
      R.f_field_eps = (float)d.field_eps;
      R.spec_base = spec;
      R.tw1_base = tw;
      R.tw2_base = tw + M1;
      R.y_base = ybuf;
      R.fna = na;
      R.fnb = nb;
      R.flist_base = flist;
      h_flist.insert(h_flist.end(), alist.begin(), alist.end());
      h_flist.insert(h_flist.end(), blist.begin(), blist.end());
      flist += na + nb;
      R.f_mpad = field_dft_mpad(d.width);
      R.f_kchunks = field_dft_kchunks(na);
      R.fa_base = fa;
      h_fa.resize(fa + (size_t)R.f_mpad * 32 * R.f_kchunks);
      build_field_dft_image(d.width, M1, alist.data(), na, R.f_mpad, R.f_kchunks, h_fa.data() + fa);
      fa += (long long)R.f_mpad * 32 * R.f_kchunks;
      R.map_base = maps;
      for (int a = 0; a < M1; a++)
        for (int b = 0; b < M2; b++)
          if (l1[a] * l2[b] / ((double)M1 * M2) < -1e-15) c->field_negative[r]++;
      // sqrt(lambda) of the kept modes, [a index][b index]
      h_spec.resize(spec + (size_t)na * nb);
      for (int j = 0; j < na; j++)
        for (int jb = 0; jb < nb; jb++) {
          const double lam = l1[alist[j]] * l2[blist[jb]] / ((double)M1 * M2);
          h_spec[spec + (size_t)j * nb + jb] = lam > 0 ? (float)std::sqrt(lam) : 0.f;
        }
      h_tw.resize(tw + M1 + M2);
      for (int k = 0; k < M1; k++)
        h_tw[tw + k] = make_float2((float)std::cos(2.0 * M_PI * k / M1), (float)-std::sin(2.0 * M_PI * k / M1));
      for (int k = 0; k < M2; k++)
        h_tw[tw + M1 + k] = make_float2((float)std::cos(2.0 * M_PI * k / M2), (float)-std::sin(2.0 * M_PI * k / M2));
      spec += (long long)na * nb;
      tw += M1 + M2;
      ybuf += (long long)d.nclones * d.width * field_y_pitch(nb);
      maps += (long long)d.nclones * R.nodes;
      c->any_field = true;
      c->field_max_w = std::max(c->field_max_w, d.width);
      c->field_max_m1 = std::max(c->field_max_m1, M1);
      c->field_max_m2 = std::max(c->field_max_m2, M2);
      c->field_max_tiles2 = std::max(c->field_max_tiles2, ((d.width + 63) / 64) * ((d.height + 63) / 64));
    }
    pop += (long long)d.nclones * 9 * R.plane;
    terms += (long long)R.nterms * d.nclones;
    if (d.perturb_mode == CLBM_PERTURB_MIX) {
      snaps += (long long)R.nsnap * 9 * R.plane;
      c->any_mix = true;
    }
    clones += d.nclones;
    blocks += d.nclones * R.blocks_per_clone;
    c->max_nodes = std::max(c->max_nodes, R.nodes);
  }
  if (clones > 65535) {
    delete c;
    return fail(CLBM_ERR_INVALID, "more than 65535 clones in one context");
  }
  c->total_clones = clones;
  c->total_blocks = blocks;
  c->pop_elems = (size_t)pop;
  c->d.term_slab = terms;
  c->d.max_steps = max_steps;
  c->d.max_intervals = 1 << 16;

  auto bail = [&](cudaError_t e) {
    int s = clbm_status_from_cuda(e);
    clbm_destroy(c);
    return s;
  };
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e);
  for (int b = 0; b < 2; b++)
    if ((e = cudaMalloc(&c->pop[b], c->pop_elems * c->elem_size)) != cudaSuccess) return bail(e);
  DevArrays &D = c->d;
  c->run_cs.assign(nruns, 0);
  c->run_tv.assign(nruns, 0);
  c->run_rows.assign(nruns, std::vector<int>());
  c->stream_nruns = nruns;
  if ((e = dalloc(c->d_runs_stream, nruns)) != cudaSuccess) return bail(e);
  if ((e = dalloc(D.runs, nruns)) != cudaSuccess) return bail(e);
  if ((e = dalloc(D.state, nruns)) != cudaSuccess) return bail(e);
  if ((e = dalloc(D.sacc, clones)) != cudaSuccess) return bail(e);
  if ((e = dalloc(D.drag, (size_t)clones * max_steps)) != cudaSuccess) return bail(e);
  if ((e = dalloc(D.weights, clones)) != cudaSuccess) return bail(e);
  if ((e = dalloc(D.labels, clones)) != cudaSuccess) return bail(e);
  if ((e = dalloc(D.mark, clones)) != cudaSuccess) return bail(e);
  if ((e = dalloc(D.copies_pre, clones)) != cudaSuccess) return bail(e);
  if ((e = dalloc(D.copies_post, clones)) != cudaSuccess) return bail(e);
  if ((e = dalloc(D.prefactors, c->any_mix ? (size_t)clones * MAX_SNAP : 1)) != cudaSuccess) return bail(e);
  if ((e = dalloc(D.pert, 2 * (size_t)clones)) != cudaSuccess) return bail(e);
  if ((e = dalloc(D.partials, c->any_mix ? 2 * (size_t)blocks : 1)) != cudaSuccess) return bail(e);
  if ((e = dalloc(D.scratch_i, 4 * (size_t)clones + 4 * (size_t)nruns)) != cudaSuccess) return bail(e);
  if ((e = dalloc(D.scratch_d, clones)) != cudaSuccess) return bail(e);
  if ((e = dalloc(D.snaps, (size_t)snaps)) != cudaSuccess) return bail(e);
  if ((e = dalloc(D.rvalues, (size_t)nruns * D.max_intervals)) != cudaSuccess) return bail(e);
  if ((e = dalloc(D.logr, (size_t)nruns * D.max_intervals)) != cudaSuccess) return bail(e);
  if ((e = dalloc(D.err, 1)) != cudaSuccess) return bail(e);
  if ((e = cudaMalloc(&D.terms, (size_t)terms * max_steps * c->elem_size)) != cudaSuccess) return bail(e);
  if ((e = dalloc(c->d_identity, clones)) != cudaSuccess) return bail(e);
  if ((e = dalloc(c->d_zeros, clones)) != cudaSuccess) return bail(e);
  if (c->any_field) {
    if ((e = dalloc(c->d_spec, (size_t)spec)) != cudaSuccess) return bail(e);
    if ((e = dalloc(c->d_tw, (size_t)tw)) != cudaSuccess) return bail(e);
    if ((e = dalloc(c->d_ybuf, (size_t)ybuf)) != cudaSuccess) return bail(e);
    if ((e = dalloc(c->d_fa, (size_t)fa)) != cudaSuccess) return bail(e);
    if ((e = dalloc(c->d_flist, (size_t)flist)) != cudaSuccess) return bail(e);
    if ((e = cudaMemcpy(c->d_flist, h_flist.data(), sizeof(int) * flist, cudaMemcpyHostToDevice)) != cudaSuccess) return bail(e);
    if ((e = cudaMemcpy(c->d_fa, h_fa.data(), sizeof(float) * fa, cudaMemcpyHostToDevice)) != cudaSuccess) return bail(e);
    if ((e = dalloc(c->d_maps, (size_t)maps)) != cudaSuccess) return bail(e);
    if ((e = cudaMemcpy(c->d_spec, h_spec.data(), sizeof(float) * spec, cudaMemcpyHostToDevice)) != cudaSuccess) return bail(e);
    if ((e = cudaMemcpy(c->d_tw, h_tw.data(), sizeof(float2) * tw, cudaMemcpyHostToDevice)) != cudaSuccess) return bail(e);
    if ((e = cudaMemset(c->d_maps, 0, sizeof(float) * maps)) != cudaSuccess) return bail(e);
  }
  if ((e = cudaMemset(c->d_zeros, 0, sizeof(int) * clones)) != cudaSuccess) return bail(e);

  std::vector<RunState> st(nruns);
  std::vector<int> ident(clones);
  for (int r = 0; r < nruns; r++) {
    RunState &s = st[r];
    memset(&s, 0, sizeof(s));
    // never-seeded glibc drand48 starts at X = 0 on every rank; rank 0 runs
    // srand(1) and discards 1000 rand() values (pops driver :176-178)
    glibc_srand(s.rnd, 1);
    for (int i = 0; i < 1000; i++) glibc_rand_next(s.rnd);
    for (int j = 0; j < runs[r].nclones; j++) ident[c->runs_h[r].clone_base + j] = j;
  }
  cudaStream_t s = c->stream;
  if ((e = cudaMemcpyAsync(D.runs, c->runs_h.data(), sizeof(RunDev) * nruns, cudaMemcpyHostToDevice, s)) != cudaSuccess) return bail(e);
  if ((e = cudaMemcpyAsync(D.state, st.data(), sizeof(RunState) * nruns, cudaMemcpyHostToDevice, s)) != cudaSuccess) return bail(e);
  if ((e = cudaMemcpyAsync(c->d_identity, ident.data(), sizeof(int) * clones, cudaMemcpyHostToDevice, s)) != cudaSuccess) return bail(e);
  if ((e = cudaMemcpyAsync(D.labels, c->d_identity, sizeof(int) * clones, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return bail(e);
  if ((e = cudaMemsetAsync(D.mark, 0, sizeof(int) * clones, s)) != cudaSuccess) return bail(e);
  if ((e = cudaMemsetAsync(D.err, 0, sizeof(unsigned), s)) != cudaSuccess) return bail(e);
  if ((e = cudaMemsetAsync(D.sacc, 0, sizeof(double) * clones, s)) != cudaSuccess) return bail(e);
  if ((e = cudaMemsetAsync(D.pert, 0, sizeof(double) * 2 * clones, s)) != cudaSuccess) return bail(e);
  for (int b = 0; b < 2; b++)
    if ((e = cudaMemsetAsync(c->pop[b], 0, c->pop_elems * c->elem_size, s)) != cudaSuccess) return bail(e);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return bail(e);
  *out = c;
  return CLBM_OK;
}

static int check_run(clbm_ctx *c, int run) {
  if (!c) return fail(CLBM_ERR_INVALID, "ctx is NULL");
  if (run < 0 || run >= c->nruns) return fail(CLBM_ERR_INVALID, "run index out of range");
  return CLBM_OK;
}

extern "C" int clbm_load_run_aos_f64(clbm_ctx *c, int run, const double *aos) {
  if (int s = check_run(c, run)) return s;
  if (!aos) return fail(CLBM_ERR_INVALID, "aos is NULL");
  const RunDev &R = c->runs_h[run];
  const bool f64 = c->precision == CLBM_FP64;
  const size_t n = 9 * (size_t)R.nodes, clone_bytes = n * 8;
  // staging: the two halves of the population buffer that does not hold the
  // current state (its content is dead until the next interval's reseed
  // writes it), copies of chunk i+1 overlapping the conversion of chunk i
  const size_t half = c->pop_elems * c->elem_size / 2;
  const int chunk = (int)std::min<size_t>(R.nclones, half / clone_bytes);
  if (chunk < 1) {  // one clone larger than half the buffer: a temporary stage
    double *stage = nullptr;
    CK(cudaMallocAsync((void **)&stage, clone_bytes, c->stream));
    cudaError_t e = cudaSuccess;
    for (int j = 0; j < R.nclones && e == cudaSuccess; j++) {
      e = cudaMemcpyAsync(stage, aos + (size_t)j * n, clone_bytes, cudaMemcpyHostToDevice, c->stream);
      if (e == cudaSuccess) e = launch_aos_to_soa(f64, c->d.runs, run, R.nodes, j, 1, stage, c->pop[c->s_buf], c->stream);
    }
    cudaFreeAsync(stage, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return clbm_status_from_cuda(e);
  }
  double *stage[2] = {(double *)c->pop[1 - c->s_buf],
                      (double *)((char *)c->pop[1 - c->s_buf] + (half & ~(size_t)255))};
  cudaStream_t conv = nullptr;
  cudaEvent_t copied[2] = {nullptr, nullptr}, converted[2] = {nullptr, nullptr};
  cudaError_t e = cudaStreamCreateWithFlags(&conv, cudaStreamNonBlocking);
  for (int b = 0; b < 2 && e == cudaSuccess; b++) {
    e = cudaEventCreateWithFlags(&copied[b], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&converted[b], cudaEventDisableTiming);
  }
  int i = 0;
  for (int c0 = 0; c0 < R.nclones && e == cudaSuccess; c0 += chunk, i++) {
    const int m = std::min(chunk, R.nclones - c0), b = i & 1;
    if (i >= 2) e = cudaStreamWaitEvent(c->stream, converted[b], 0);  // chunk i-2 has left this half
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(stage[b], aos + (size_t)c0 * n, clone_bytes * m, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaEventRecord(copied[b], c->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(conv, copied[b], 0);
    if (e == cudaSuccess) e = launch_aos_to_soa(f64, c->d.runs, run, R.nodes, c0, m, stage[b], c->pop[c->s_buf], conv);
    if (e == cudaSuccess) e = cudaEventRecord(converted[b], conv);
  }
  if (conv) {
    const cudaError_t e2 = cudaStreamSynchronize(conv);
    if (e == cudaSuccess) e = e2;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  for (int b = 0; b < 2; b++) {
    if (copied[b]) cudaEventDestroy(copied[b]);
    if (converted[b]) cudaEventDestroy(converted[b]);
  }
  if (conv) cudaStreamDestroy(conv);
  return clbm_status_from_cuda(e);
}

extern "C" int clbm_load_pops_aos_f64(clbm_ctx *c, int run, int clone, const double *aos) {
  if (int s = check_run(c, run)) return s;
  const RunDev &R = c->runs_h[run];
  if (clone < 0 || clone >= R.nclones || !aos) return fail(CLBM_ERR_INVALID, "bad clone or NULL array");
  const size_t n = 9 * (size_t)R.nodes;
  double *stage = nullptr;
  CK(cudaMallocAsync((void **)&stage, n * 8, c->stream));
  cudaError_t e = cudaMemcpyAsync(stage, aos, n * 8, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess)
    e = launch_aos_to_soa(c->precision == CLBM_FP64, c->d.runs, run, R.nodes, clone, 1, stage, c->pop[c->s_buf], c->stream);
  cudaFreeAsync(stage, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return clbm_status_from_cuda(e);
}

extern "C" int clbm_dump_pops_aos_f64(clbm_ctx *c, int run, int clone, double *aos) {
  if (int s = check_run(c, run)) return s;
  const RunDev &R = c->runs_h[run];
  if (clone < 0 || clone >= R.nclones || !aos) return fail(CLBM_ERR_INVALID, "bad clone or NULL array");
  int parent = clone;
  CK(cudaMemcpyAsync(&parent, c->d.labels + R.clone_base + clone, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (parent < 0 || parent >= R.nclones) return fail(CLBM_ERR_DEVICE, "corrupt pending label");
  const size_t n = 9 * (size_t)R.nodes;
  double *stage = nullptr;
  CK(cudaMallocAsync((void **)&stage, n * 8, c->stream));
  cudaError_t e = launch_soa_to_aos(c->precision == CLBM_FP64, c->d.runs, run, R.nodes, parent, c->pop[c->s_buf], stage, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(aos, stage, n * 8, cudaMemcpyDeviceToHost, c->stream);
  cudaFreeAsync(stage, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return clbm_status_from_cuda(e);
}

extern "C" int clbm_set_snapshots_aos_f64(clbm_ctx *c, int run, int nsnap, const double *aos) {
  if (int s = check_run(c, run)) return s;
  const RunDev &R = c->runs_h[run];
  if (R.perturb_mode != CLBM_PERTURB_MIX) return fail(CLBM_ERR_INVALID, "run does not use the snapshot mix");
  if (nsnap != R.nsnap || !aos) return fail(CLBM_ERR_INVALID, "nsnap differs from the run descriptor");
  const size_t n = 9 * (size_t)R.nodes * nsnap;
  double *stage = nullptr;
  CK(cudaMallocAsync((void **)&stage, n * 8, c->stream));
  cudaError_t e = cudaMemcpyAsync(stage, aos, n * 8, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = launch_snaps_to_soa(c->d.runs, run, R.nodes, nsnap, stage, c->d.snaps, c->stream);
  cudaFreeAsync(stage, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) c->snaps_loaded[run] = 1;
  return clbm_status_from_cuda(e);
}

extern "C" int clbm_init_equilibrium(clbm_ctx *c, int run, double u0, double noise,
                                     unsigned long long seed) {
  if (int s = check_run(c, run)) return s;
  cudaError_t e = launch_init_equilibrium(c->precision == CLBM_FP64, c->d.runs, c->nruns, run,
                                          c->pop[c->s_buf], u0, noise, seed, 0, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return clbm_status_from_cuda(e);
}

// ---------------------------------------------------------------------------
// The LB steps of an interval under a plan: which runs the streaming step
// kernel advances (through which descriptor table) and which run
// cluster-resident, with which cluster size and thread count.
struct LbPlan {
  std::vector<int> cs, tv;        // per run: cluster size (0 = streaming), thread variant
  std::vector<std::vector<int>> rows;  // per run: band split row0[0..cs] (empty = even)
  std::vector<char> active;       // runs to advance (autotuner timing of one run); empty = all
  const RunDev *table = nullptr;  // step-kernel table of the streaming runs
  int nstream = 0, tiles[3] = {0, 0, 0}, variant = 0;
};

static bool plan_active(const LbPlan &p, int r) { return p.active.empty() || p.active[r]; }

static LbPlan current_plan(const clbm_ctx *c, bool f64) {
  LbPlan p;
  p.cs = f64 ? std::vector<int>(c->nruns, 0) : c->run_cs;
  p.tv = c->run_tv;
  p.rows = c->run_rows;
  const bool sub = !f64 && c->stream_subset;
  p.table = sub ? c->d_runs_stream : c->d.runs;
  p.nstream = sub ? c->stream_nruns : c->nruns;
  for (int q = 0; q < 3; q++) p.tiles[q] = sub ? c->stream_tiles[q] : c->total_tiles[q];
  p.variant = c->step_variant;
  return p;
}

// The streaming runs' own step-kernel table: their descriptors with tile
// bases counted over these runs only (the grid covers just their tiles).
static cudaError_t upload_stream_table(clbm_ctx *c, const std::vector<int> &runs) {
  c->stream_h.clear();
  int tiles[3] = {0, 0, 0};
  for (int r : runs) {
    RunDev R = c->runs_h[r];
    for (int q = 0; q < 3; q++) {
      R.tile_base[q] = tiles[q];
      tiles[q] += R.nclones * R.tiles[q];
    }
    c->stream_h.push_back(R);
  }
  for (int q = 0; q < 3; q++) c->stream_tiles[q] = tiles[q];
  c->stream_nruns = (int)runs.size();
  if (runs.empty()) return cudaSuccess;
  // pageable source: the copy is staged before the call returns
  return cudaMemcpyAsync(c->d_runs_stream, c->stream_h.data(), sizeof(RunDev) * runs.size(),
                         cudaMemcpyHostToDevice, c->stream);
}

static cudaError_t ensure_side(clbm_ctx *c, int n) {
  while ((int)c->side.size() < n) {
    cudaStream_t t = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&t, cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
    c->side.push_back(t);
  }
  while ((int)c->fork_join.size() < n + 1) {
    cudaEvent_t ev = nullptr;
    cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) return e;
    c->fork_join.push_back(ev);
  }
  return cudaSuccess;
}

// Enqueue `steps` LB steps of the plan's runs.  Interval: P_0 in buffer src,
// S_T left in buffer dst; the streaming runs alternate between the two
// buffers as the pull scheme does and store S on their last step.  timing
// (autotuner): every streaming launch reads src and writes the other buffer
// and none is a last step, so the state in src is left untouched.  fuse
// (cluster-resident runs only): the kernels form P_0 themselves from the
// reseed's inputs (fuse->src, a buffer other than dst) instead of reading src.
static cudaError_t enqueue_lb_steps(clbm_ctx *c, const LbPlan &p, int steps, int src, int dst, bool timing,
                                    const ReseedArgs *fuse = nullptr) {
  const bool f64 = c->precision == CLBM_FP64;
  cudaStream_t s = c->stream;
  cudaError_t e;
  int nside = 0;
  for (int r = 0; r < c->nruns; r++) nside += p.cs[r] > 0 && plan_active(p, r);
  if (nside) {
    if ((e = ensure_side(c, nside)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(c->fork_join[0], s)) != cudaSuccess) return e;
  }
  int i = 0;
  for (int r = 0; r < c->nruns; r++) {
    if (!(p.cs[r] > 0 && plan_active(p, r))) continue;
    const RunDev &R = c->runs_h[r];
    cudaStream_t ts = c->side[i];
    if ((e = cudaStreamWaitEvent(ts, c->fork_join[0], 0)) != cudaSuccess) return e;
    TemporalArgs ta{R, r, steps, (const float *)c->pop[src], (float *)c->pop[dst], (float *)c->d.terms,
                    c->d.term_slab, c->d.err, c->d_maps, {}, fuse ? 1 : 0, fuse ? *fuse : ReseedArgs{}};
    const int cs = p.cs[r];
    if (r < (int)p.rows.size() && (int)p.rows[r].size() == cs + 1)
      std::copy(p.rows[r].begin(), p.rows[r].end(), ta.band_row0);
    else
      even_band_rows(R.H, cs, ta.band_row0);
    if ((e = launch_temporal(ta, cs, p.tv[r], R.nclones, R.W, ts)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(c->fork_join[1 + i], ts)) != cudaSuccess) return e;
    i++;
  }
  if (p.nstream > 0) {
    int cur = src;
    for (int t = 0; t < steps; t++) {
      StepArgs a{p.table, p.nstream, t, c->pop[cur], c->pop[1 - cur], c->d.terms, c->d.term_slab,
                 c->d.err, c->total_clones, c->max_nodes, {p.tiles[0], p.tiles[1], p.tiles[2]}, c->d_maps};
      if ((e = launch_step(f64, !timing && t == steps - 1, a, c->total_blocks, s, p.variant)) != cudaSuccess)
        return e;
      if (!timing) cur = 1 - cur;
    }
  }
  for (int k = 0; k < nside; k++)
    if ((e = cudaStreamWaitEvent(s, c->fork_join[1 + k], 0)) != cudaSuccess) return e;
  return cudaSuccess;
}

// Install a plan: per run cluster size (0 = streaming), thread variant and
// band split (empty: even), the streaming runs' launch variant.  Captured
// intervals are dropped.
static cudaError_t set_plan(clbm_ctx *c, const std::vector<int> &cs, const std::vector<int> &tv, int variant,
                            const std::vector<std::vector<int>> &rows = {}) {
  c->run_cs = cs;
  c->run_tv = tv;
  c->run_rows = rows;
  c->run_rows.resize(c->nruns);
  c->step_variant = variant;
  std::vector<int> streaming;
  for (int r = 0; r < c->nruns; r++)
    if (!cs[r]) streaming.push_back(r);
  c->stream_subset = (int)streaming.size() != c->nruns;
  cudaError_t e = cudaSuccess;
  if (c->stream_subset)
    e = upload_stream_table(c, streaming);
  else
    c->stream_nruns = c->nruns;
  destroy_graphs(c);
  return e;
}

// Enqueue one interval on the context's stream (no synchronisation).
// prof: record an event pair around the step launches (eager mode only).
static cudaError_t enqueue_interval(clbm_ctx *c, int steps, int sbuf, bool prof = false) {
  const bool f64 = c->precision == CLBM_FP64;
  cudaStream_t s = c->stream;
  cudaError_t e;
  const void *S = c->pop[sbuf];
  if (c->any_mix) {
    e = launch_perturb_norms(f64, c->d.runs, c->nruns, S, c->d.labels, c->d.mark, c->d.prefactors,
                             c->d.snaps, c->d.partials, c->d.pert, c->total_blocks, c->total_clones, s);
    if (e != cudaSuccess) return e;
  }
  if (c->any_field) {
    if (prof) {  // an event pair around the field kernels
      while ((size_t)c->fev_used + 2 > c->fev.size()) {
        cudaEvent_t ne;
        if ((e = cudaEventCreate(&ne)) != cudaSuccess) return e;
        c->fev.push_back(ne);
      }
      if ((e = cudaEventRecord(c->fev[c->fev_used], s)) != cudaSuccess) return e;
    }
    FieldArgs fa{c->d.runs, c->nruns, c->d.state, c->d_spec, c->d_tw, c->d_ybuf, c->d_maps, c->d_fa, c->d.err, c->d_flist};
    e = launch_fields(fa, c->total_clones, c->field_max_w, c->field_max_m1, c->field_max_m2,
                      c->field_max_tiles2, s);
    if (e != cudaSuccess) return e;
    if (prof) {
      if ((e = cudaEventRecord(c->fev[c->fev_used + 1], s)) != cudaSuccess) return e;
      c->fev_used += 2;
    }
  }
  ReseedArgs ra{c->d.runs, c->nruns, S, c->pop[1 - sbuf], c->d.labels, c->d.mark, c->d.pert,
                c->d.prefactors, c->d.snaps, c->d.state, c->d.err, c->d_maps};
  const LbPlan plan = current_plan(c, f64);
  // Every run cluster-resident under the uniform body force and an even step
  // count (S_T then goes to the other buffer than S): the interval kernels do
  // the reseed while loading their clones, which saves writing P_0 and
  // reading it back.  (With an odd count S_T would overwrite S while other
  // clusters still copy parents.)
  bool fuse = !f64 && !c->any_field && steps % 2 == 0;
  for (int r = 0; r < c->nruns; r++) fuse = fuse && plan.cs[r] > 0;
  if (!fuse && (e = launch_reseed(f64, ra, c->total_blocks, s)) != cudaSuccess) return e;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (prof) {
    if ((size_t)c->ev_used + 2 > c->ev.size()) {
      for (int i = 0; i < 2; i++) {
        cudaEvent_t ne;
        if ((e = cudaEventCreate(&ne)) != cudaSuccess) return e;
        c->ev.push_back(ne);
      }
    }
    e0 = c->ev[c->ev_used];
    e1 = c->ev[c->ev_used + 1];
    c->ev_used += 2;
    c->prof_steps += steps;
    if ((e = cudaEventRecord(e0, s)) != cudaSuccess) return e;
  }
  // P_0 (the reseed output) is in 1 - sbuf; S_T goes where the streaming
  // sequence leaves it.  Cluster-resident runs: the whole interval on chip,
  // one launch each on its own side stream; the streaming runs meanwhile one
  // step launch per step on the main stream; the side streams join before the
  // drag reduction (a captured interval holds them as parallel branches).
  if ((e = enqueue_lb_steps(c, plan, steps, 1 - sbuf, (steps % 2 == 1) ? sbuf : 1 - sbuf, false,
                            fuse ? &ra : nullptr)) != cudaSuccess)
    return e;
  if (prof && (e = cudaEventRecord(e1, s)) != cudaSuccess) return e;
  if ((e = launch_drag_reduce(f64, c->d, c->nruns, c->total_clones, steps, c->any_stress, c->any_momentum, s)) != cudaSuccess) return e;
  if (c->hist_max > 0) {
    if (c->hist_steps == 0) c->hist_steps = steps;
    if (c->hist_steps != steps) c->hist_steps_varied = true;
    if ((e = launch_hist_drag(c->d, c->total_clones, steps, c->hist_drag, c->hist_max, s)) != cudaSuccess)
      return e;
  }
  // the pending copies and perturbations have been applied
  if ((e = cudaMemcpyAsync(c->d.labels, c->d_identity, sizeof(int) * c->total_clones,
                           cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
    return e;
  return cudaMemsetAsync(c->d.mark, 0, sizeof(int) * c->total_clones, s);
}

static int check_snapshots(clbm_ctx *c) {
  for (int r = 0; r < c->nruns; r++)
    if (c->runs_h[r].perturb_mode == CLBM_PERTURB_MIX && !c->snaps_loaded[r])
      return fail(CLBM_ERR_INVALID, "snapshot-mix run without snapshots (clbm_set_snapshots_aos_f64)");
  return CLBM_OK;
}

static int sbuf_after(int sbuf, int steps) {
  // reseed writes P into 1-sbuf and step t writes into sbuf when t is even,
  // 1-sbuf when t is odd; the last step (t = steps-1) writes S
  return (steps % 2 == 1) ? sbuf : 1 - sbuf;
}

extern "C" int clbm_run_interval(clbm_ctx *c, int steps) {
  if (!c) return fail(CLBM_ERR_INVALID, "ctx is NULL");
  if (steps < 1 || steps > c->max_steps) return fail(CLBM_ERR_INVALID, "steps outside [1, max_steps]");
  if (int st = check_snapshots(c)) return st;
  CK(enqueue_interval(c, steps, c->s_buf, c->profiling));
  c->s_buf = sbuf_after(c->s_buf, steps);
  c->last_steps = steps;
  c->pending = false;
  return CLBM_OK;
}

static cudaError_t enqueue_clone(clbm_ctx *c) {
  cudaError_t e = launch_clone(c->d, c->nruns, c->stream);
  if (e == cudaSuccess && c->hist_max > 0)
    e = launch_hist_labels(c->d, c->total_clones, c->hist_labels, c->hist_max, c->stream);
  return e;
}

static int check_error_word(clbm_ctx *c) {
  unsigned w = 0;
  CK(cudaMemcpyAsync(&w, c->d.err, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (w) {
    char msg[96];
    snprintf(msg, sizeof msg, "device error word 0x%x", w);
    return fail(CLBM_ERR_DEVICE, msg);
  }
  return CLBM_OK;
}

extern "C" int clbm_clone_step(clbm_ctx *c) {
  if (!c) return fail(CLBM_ERR_INVALID, "ctx is NULL");
  if (c->last_steps < 1) return fail(CLBM_ERR_INVALID, "clone step before any interval");
  CK(enqueue_clone(c));
  c->pending = true;
  return check_error_word(c);
}

extern "C" int clbm_get_drag(clbm_ctx *c, int run, double *out) {
  if (int s = check_run(c, run)) return s;
  if (!out) return fail(CLBM_ERR_INVALID, "out is NULL");
  if (c->last_steps < 1) return fail(CLBM_ERR_INVALID, "no interval has run");
  const RunDev &R = c->runs_h[run];
  CK(cudaMemcpy2DAsync(out, sizeof(double) * c->last_steps, c->d.drag + (size_t)R.clone_base * c->max_steps,
                       sizeof(double) * c->max_steps, sizeof(double) * c->last_steps, R.nclones,
                       cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return CLBM_OK;
}

extern "C" int clbm_get_rvalues(clbm_ctx *c, int run, int first, int count, double *rvalues,
                                double *log_rvalues) {
  if (int s = check_run(c, run)) return s;
  int done = 0;
  CK(cudaMemcpyAsync(&done, &c->d.state[run].interval, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (first < 0 || count < 0 || first + count > done || first + count > c->d.max_intervals)
    return fail(CLBM_ERR_INVALID, "requested intervals outside the recorded history");
  const size_t off = (size_t)run * c->d.max_intervals + first;
  if (rvalues && count)
    CK(cudaMemcpyAsync(rvalues, c->d.rvalues + off, sizeof(double) * count, cudaMemcpyDeviceToHost, c->stream));
  if (log_rvalues && count)
    CK(cudaMemcpyAsync(log_rvalues, c->d.logr + off, sizeof(double) * count, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return CLBM_OK;
}

extern "C" int clbm_intervals_done(clbm_ctx *c, int run, int *done) {
  if (int s = check_run(c, run)) return s;
  if (!done) return fail(CLBM_ERR_INVALID, "done is NULL");
  CK(cudaMemcpyAsync(done, &c->d.state[run].interval, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return CLBM_OK;
}

extern "C" int clbm_get_clone_result(clbm_ctx *c, int run, int *labels, double *rvalue,
                                     double *weights, int *copies_pre, int *copies_post) {
  if (int s = check_run(c, run)) return s;
  const RunDev &R = c->runs_h[run];
  const size_t nc = R.nclones, g0 = R.clone_base;
  cudaStream_t s = c->stream;
  if (labels) CK(cudaMemcpyAsync(labels, c->d.labels + g0, nc * sizeof(int), cudaMemcpyDeviceToHost, s));
  if (weights) CK(cudaMemcpyAsync(weights, c->d.weights + g0, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (copies_pre) CK(cudaMemcpyAsync(copies_pre, c->d.copies_pre + g0, nc * sizeof(int), cudaMemcpyDeviceToHost, s));
  if (copies_post) CK(cudaMemcpyAsync(copies_post, c->d.copies_post + g0, nc * sizeof(int), cudaMemcpyDeviceToHost, s));
  if (rvalue) CK(cudaMemcpyAsync(rvalue, &c->d.state[run].rbar, sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return CLBM_OK;
}

static int graph_for(clbm_ctx *c, int steps, int sbuf, cudaGraphExec_t *exec) {
  for (auto &g : c->graphs)
    if (g.exec && g.sbuf == sbuf && g.steps == steps) {
      *exec = g.exec;
      return CLBM_OK;
    }
  cudaGraph_t graph = nullptr;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = enqueue_interval(c, steps, sbuf);
  if (e == cudaSuccess) e = enqueue_clone(c);
  cudaError_t e2 = cudaStreamEndCapture(c->stream, &graph);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return clbm_status_from_cuda(e);
  }
  cudaGraphExec_t ge = nullptr;
  e = cudaGraphInstantiate(&ge, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return clbm_status_from_cuda(e);
  GraphEntry *slot = nullptr;
  for (auto &g : c->graphs)
    if (!g.exec) {
      slot = &g;
      break;
    }
  if (!slot) {
    destroy_graphs(c);
    slot = &c->graphs[0];
  }
  slot->exec = ge;
  slot->sbuf = sbuf;
  slot->steps = steps;
  *exec = ge;
  return CLBM_OK;
}

static int enqueue_sampler_interval(clbm_ctx *c, int steps);
static int copy_rvalues(clbm_ctx *c, int intervals, double *rvalues);

extern "C" int clbm_run_sampler(clbm_ctx *c, int steps, int intervals, double *rvalues) {
  if (!c) return fail(CLBM_ERR_INVALID, "ctx is NULL");
  if (steps < 1 || steps > c->max_steps || intervals < 0) return fail(CLBM_ERR_INVALID, "bad steps/intervals");
  if (int st = check_snapshots(c)) return st;
  for (int i = 0; i < intervals; i++)
    if (int st = enqueue_sampler_interval(c, steps)) return st;
  if (int st = check_error_word(c)) return st;
  if (rvalues && intervals > 0) return copy_rvalues(c, intervals, rvalues);
  return CLBM_OK;
}

// One interval (and its cloning step) on the context's stream: a CUDA graph
// under CLBM_FLAG_GRAPH (eager while profiling), else launch by launch.
static int enqueue_sampler_interval(clbm_ctx *c, int steps) {
  if ((c->flags & CLBM_FLAG_GRAPH) && !c->profiling) {
    cudaGraphExec_t ge = nullptr;
    if (int st = graph_for(c, steps, c->s_buf, &ge)) return st;
    CK(cudaGraphLaunch(ge, c->stream));
  } else {
    CK(enqueue_interval(c, steps, c->s_buf, c->profiling));
    CK(enqueue_clone(c));
  }
  c->s_buf = sbuf_after(c->s_buf, steps);
  c->last_steps = steps;
  c->pending = true;
  return CLBM_OK;
}

// R_t of the last `intervals` intervals of every run ([run][interval]).
static int copy_rvalues(clbm_ctx *c, int intervals, double *rvalues) {
  for (int r = 0; r < c->nruns; r++) {
    int f = 0;
    CK(cudaMemcpyAsync(&f, &c->d.state[r].interval, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    f -= intervals;
    if (f < 0 || f + intervals > c->d.max_intervals) return fail(CLBM_ERR_INVALID, "R_t history capacity exceeded");
    CK(cudaMemcpyAsync(rvalues + (size_t)r * intervals, c->d.rvalues + (size_t)r * c->d.max_intervals + f,
                       sizeof(double) * intervals, cudaMemcpyDeviceToHost, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  return CLBM_OK;
}

extern "C" int clbm_run_sampler_outputs(clbm_ctx *c, int steps, int intervals, double *rvalues, double *drag,
                                        int *labels, double *weights) {
  if (!c) return fail(CLBM_ERR_INVALID, "ctx is NULL");
  if (steps < 1 || steps > c->max_steps || intervals < 0) return fail(CLBM_ERR_INVALID, "bad steps/intervals");
  if (int st = check_snapshots(c)) return st;
  const size_t nc = (size_t)c->total_clones;
  for (int k = 0; k < 2; k++) {
    if (!c->h_drag[k]) CK(cudaHostAlloc((void **)&c->h_drag[k], sizeof(double) * nc * c->max_steps, cudaHostAllocDefault));
    if (!c->h_weights[k]) CK(cudaHostAlloc((void **)&c->h_weights[k], sizeof(double) * nc, cudaHostAllocDefault));
    if (!c->h_labels[k]) CK(cudaHostAlloc((void **)&c->h_labels[k], sizeof(int) * nc, cudaHostAllocDefault));
    if (!c->h_ready[k]) CK(cudaEventCreateWithFlags(&c->h_ready[k], cudaEventDisableTiming));
  }
  // interval i's outputs: device -> staging slot i % 2 right after the
  // interval (stream order: before interval i + 1 overwrites them), then,
  // once interval i + 1 is enqueued, staging -> the caller's arrays on the
  // host while the device runs it
  auto deliver = [&](int i) -> int {
    const int k = i & 1;
    CK(cudaEventSynchronize(c->h_ready[k]));
    if (drag) std::memcpy(drag + (size_t)i * nc * steps, c->h_drag[k], sizeof(double) * nc * steps);
    if (labels) std::memcpy(labels + (size_t)i * nc, c->h_labels[k], sizeof(int) * nc);
    if (weights) std::memcpy(weights + (size_t)i * nc, c->h_weights[k], sizeof(double) * nc);
    return CLBM_OK;
  };
  for (int i = 0; i < intervals; i++) {
    if (int st = enqueue_sampler_interval(c, steps)) return st;
    const int k = i & 1;
    cudaStream_t s = c->stream;
    if (drag)
      CK(cudaMemcpy2DAsync(c->h_drag[k], sizeof(double) * steps, c->d.drag, sizeof(double) * c->max_steps,
                           sizeof(double) * steps, nc, cudaMemcpyDeviceToHost, s));
    if (labels) CK(cudaMemcpyAsync(c->h_labels[k], c->d.labels, sizeof(int) * nc, cudaMemcpyDeviceToHost, s));
    if (weights) CK(cudaMemcpyAsync(c->h_weights[k], c->d.weights, sizeof(double) * nc, cudaMemcpyDeviceToHost, s));
    CK(cudaEventRecord(c->h_ready[k], s));
    if (i > 0)
      if (int st = deliver(i - 1)) return st;
  }
  if (intervals > 0)
    if (int st = deliver(intervals - 1)) return st;
  if (int st = check_error_word(c)) return st;
  if (rvalues && intervals > 0) return copy_rvalues(c, intervals, rvalues);
  return CLBM_OK;
}

extern "C" int clbm_error_word(clbm_ctx *c, unsigned *word, int clear) {
  if (!c || !word) return fail(CLBM_ERR_INVALID, "NULL argument");
  CK(cudaMemcpyAsync(word, c->d.err, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  if (clear) CK(cudaMemsetAsync(c->d.err, 0, sizeof(unsigned), c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return CLBM_OK;
}

extern "C" int clbm_sync(clbm_ctx *c) {
  if (!c) return fail(CLBM_ERR_INVALID, "ctx is NULL");
  CK(cudaStreamSynchronize(c->stream));
  return CLBM_OK;
}

extern "C" void *clbm_stream(clbm_ctx *c) { return c ? (void *)c->stream : nullptr; }

extern "C" int clbm_profile(clbm_ctx *c, int enable) {
  if (!c) return fail(CLBM_ERR_INVALID, "ctx is NULL");
  c->profiling = enable != 0;
  c->ev_used = 0;
  c->prof_steps = 0;
  c->fev_used = 0;
  return CLBM_OK;
}

extern "C" int clbm_profile_read(clbm_ctx *c, double *step_ms, int *nsteps) {
  if (!c || !step_ms || !nsteps) return fail(CLBM_ERR_INVALID, "NULL argument");
  CK(cudaStreamSynchronize(c->stream));
  double total = 0.0;
  for (int i = 0; i + 1 < c->ev_used; i += 2) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->ev[i], c->ev[i + 1]));
    total += ms;
  }
  *step_ms = total;
  *nsteps = c->prof_steps;
  c->ev_used = 0;
  c->prof_steps = 0;
  return CLBM_OK;
}

extern "C" int clbm_profile_read_fields(clbm_ctx *c, double *field_ms, int *nintervals) {
  if (!c || !field_ms || !nintervals) return fail(CLBM_ERR_INVALID, "NULL argument");
  CK(cudaStreamSynchronize(c->stream));
  double total = 0.0;
  for (int i = 0; i + 1 < c->fev_used; i += 2) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->fev[i], c->fev[i + 1]));
    total += ms;
  }
  *field_ms = total;
  *nintervals = c->fev_used / 2;
  c->fev_used = 0;
  return CLBM_OK;
}

// Variant numbering: 0 .. step_variant_count()-1 are the streaming step
// launches; after them, for each cluster size of kClusterSizes in that order,
// the cluster-resident interval kernel's thread configurations.  The sizes
// that are not powers of two come last, so the numbers of the others do not
// move.  The GPCs' SM counts set how many clusters of a size are resident
// (one CTA per SM, GB300's 152 SMs): 2 -> 152 SMs busy, 3 -> 138, 4 -> 144,
// 5 -> 140, 6 -> 138, 7 -> 105, 8 -> 120, 9 -> 135, 10 -> 130, 11 to 16 ->
// 88 to 112; 9 and 10 serve lattices too large for 8 CTAs' shared memory.
static const int kClusterSizes[] = {1, 2, 4, 8, 16, 3, 5, 6, 7, 9, 10};
static constexpr int kNumClusterSizes = (int)(sizeof(kClusterSizes) / sizeof(kClusterSizes[0]));

static int variant_count() { return step_variant_count() + kNumClusterSizes * temporal_variant_count(); }

static void variant_shape(int v, int &cs, int &tv) {
  const int nv = step_variant_count();
  cs = 0;
  tv = 0;
  if (v >= nv && v < variant_count()) {
    const int q = v - nv;
    cs = kClusterSizes[q / temporal_variant_count()];
    tv = q % temporal_variant_count();
  }
}

static int variant_index(int cs, int tv) {
  for (int j = 0; cs && j < kNumClusterSizes; j++)
    if (kClusterSizes[j] == cs) return step_variant_count() + j * temporal_variant_count() + tv;
  return 0;
}

// whether run r's lattice can run cluster-resident at this shape (even split)
static bool shape_fits(const RunDev &R, int cs, int tv) {
  return R.H >= cs && cs <= MAX_CLUSTER &&
         temporal_max_clusters(cs, tv, R.W, (R.H + cs - 1) / cs, R.field_mode != 0) >= 1;
}

// largest band of a split row0[0..cs]
static int split_rows_max(const std::vector<int> &row0) {
  int m = 0;
  for (size_t b = 0; b + 1 < row0.size(); b++) m = std::max(m, row0[b + 1] - row0[b]);
  return m;
}

// Weights of the general path the autotuner balances band splits for.
static const double kBalanceGamma[] = {0.5, 1.0, 1.5, 2.0, 3.0, 4.0, 6.0, 8.0};

// Run R's band split at cluster size cs balanced for weight gamma, if it
// differs from the even split and the shape stays resident at thread
// variant tv; else empty.
static std::vector<int> balanced_split(const RunDev &R, int cs, int tv, double gamma) {
  std::vector<int> even(cs + 1), row0(cs + 1);
  even_band_rows(R.H, cs, even.data());
  if (!balanced_band_rows(R.W, R.H, R.xmin, R.xmax, R.ymin, R.ymax, cs, gamma, temporal_rows_limit(R.W),
                          row0.data()) ||
      row0 == even || temporal_max_clusters(cs, tv, R.W, split_rows_max(row0), R.field_mode != 0) < 1)
    return {};
  return row0;
}

// one variant for every run
static cudaError_t apply_variant(clbm_ctx *c, int v) {
  int cs, tv;
  variant_shape(v, cs, tv);
  return set_plan(c, std::vector<int>(c->nruns, cs), std::vector<int>(c->nruns, tv),
                  cs ? c->step_variant : v);
}

// Milliseconds per LB step of a plan on this context's workload, at an
// interval boundary: timing mode reads the state and writes only the idle
// buffer, so the sampler is untouched.  One short warm-up pass first.
static cudaError_t time_plan(clbm_ctx *c, const LbPlan &p, int steps, cudaEvent_t e0, cudaEvent_t e1,
                             double *ms_per_step) {
  cudaError_t e = enqueue_lb_steps(c, p, 1, c->s_buf, 1 - c->s_buf, true);
  if (e == cudaSuccess) e = cudaEventRecord(e0, c->stream);
  if (e == cudaSuccess) e = enqueue_lb_steps(c, p, steps, c->s_buf, 1 - c->s_buf, true);
  if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  *ms_per_step = ms / steps;
  return e;
}

// A plan over every run with the streaming runs (cs == 0) in their own table.
static cudaError_t full_plan(clbm_ctx *c, const std::vector<int> &cs, const std::vector<int> &tv, int sv,
                             LbPlan &p) {
  p = LbPlan{};
  p.cs = cs;
  p.tv = tv;
  p.variant = sv;
  std::vector<int> streaming;
  for (int r = 0; r < c->nruns; r++)
    if (!cs[r]) streaming.push_back(r);
  if ((int)streaming.size() == c->nruns) {
    p.table = c->d.runs;
    p.nstream = c->nruns;
    for (int q = 0; q < 3; q++) p.tiles[q] = c->total_tiles[q];
    return cudaSuccess;
  }
  cudaError_t e = upload_stream_table(c, streaming);
  p.table = c->d_runs_stream;
  p.nstream = c->stream_nruns;
  for (int q = 0; q < 3; q++) p.tiles[q] = c->stream_tiles[q];
  return e;
}

// Autotuner: time the candidates on this context's own workload and keep the
// fastest.  Uniform candidates first (every run on one variant: the 8
// streaming launch shapes, then each cluster-resident shape that fits every
// lattice).  With several runs, each run's own best is then found alone
// (the best streaming shape against every cluster-resident shape that fits
// it), and that per-run plan -- cluster-resident runs concurrent with the
// streaming ones -- is timed as a whole and kept if it beats the uniform
// winner.  Results are cached per (lattice sizes, clone counts) for the
// process.
#include <map>
#include <mutex>
struct TuneResult {
  int best;
  std::vector<int> cs, tv;
  int sv;
  std::vector<std::vector<int>> rows;
};
static std::mutex g_tune_mutex;
static std::map<std::vector<long long>, TuneResult> g_tune_cache;

extern "C" int clbm_autotune(clbm_ctx *c, int launches, int *best, double *ms_per_variant,
                             int *nvariants) {
  if (!c) return fail(CLBM_ERR_INVALID, "ctx is NULL");
  const int nv = step_variant_count(), ntv = temporal_variant_count();
  if (nvariants) *nvariants = variant_count();
  if (c->precision != CLBM_FP32) {
    if (best) *best = 0;
    return CLBM_OK;
  }
  std::vector<long long> key;
  for (const RunDev &R : c->runs_h) {
    key.push_back(R.W);
    key.push_back(R.H);
    key.push_back(R.nclones);
  }
  if (!ms_per_variant) {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      CK(set_plan(c, it->second.cs, it->second.tv, it->second.sv, it->second.rows));
      if (best) *best = it->second.best;
      return CLBM_OK;
    }
  }
  if (launches < 1) launches = 5;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  auto bail = [&](cudaError_t e) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return clbm_status_from_cuda(e);
  };
  const int R = c->nruns;
  int arg = 0, best_sv = 0;
  double best_ms = 1e30, best_stream_ms = 1e30;
  // uniform streaming launch shapes (one launch per step)
  for (int v = 0; v < nv; v++) {
    LbPlan p;
    cudaError_t e = full_plan(c, std::vector<int>(R, 0), std::vector<int>(R, 0), v, p);
    double per = 0.0;
    if (e == cudaSuccess) e = time_plan(c, p, launches, e0, e1, &per);
    if (e != cudaSuccess) return bail(e);
    if (ms_per_variant) ms_per_variant[v] = per;
    if (per < best_stream_ms) {
      best_stream_ms = per;
      best_sv = v;
    }
  }
  best_ms = best_stream_ms;
  arg = best_sv;
  std::vector<int> plan_cs(R, 0), plan_tv(R, 0);
  std::vector<std::vector<int>> plan_rows(R);
  std::vector<std::pair<double, int>> shapes;  // (ms per step, variant) of the cluster-resident shapes
  // uniform cluster-resident shapes, timed per step over a full-length
  // interval (their HBM load and store are amortised over the steps)
  const int tsteps = std::min(c->max_steps, 100);
  for (const int cs : kClusterSizes) {
    for (int tv = 0; tv < ntv; tv++) {
      const int vidx = variant_index(cs, tv);
      if (ms_per_variant) ms_per_variant[vidx] = -1.0;
      bool ok = true;
      for (const RunDev &Rr : c->runs_h) ok = ok && shape_fits(Rr, cs, tv);
      if (!ok) continue;
      LbPlan p;
      cudaError_t e = full_plan(c, std::vector<int>(R, cs), std::vector<int>(R, tv), best_sv, p);
      double per = 0.0;
      if (e == cudaSuccess) e = time_plan(c, p, tsteps, e0, e1, &per);
      if (e != cudaSuccess) {  // this shape cannot run here: skip it
        cudaGetLastError();
        continue;
      }
      if (ms_per_variant) ms_per_variant[vidx] = per;
      shapes.emplace_back(per, vidx);
      if (per < best_ms) {
        best_ms = per;
        arg = vidx;
        plan_cs.assign(R, cs);
        plan_tv.assign(R, tv);
      }
    }
  }
  // balanced band splits of the fastest cluster-resident shapes (up to three,
  // within 25 % of the fastest): the band holding the square's box, and the
  // wall bands, carry more work per row than the others, and every step waits
  // for the slowest band
  std::sort(shapes.begin(), shapes.end());
  for (size_t q = 0; q < shapes.size() && q < 3 && shapes[q].first <= 1.25 * shapes[0].first; q++) {
    int cs, tv;
    variant_shape(shapes[q].second, cs, tv);
    for (double g : kBalanceGamma) {
      std::vector<std::vector<int>> rows(R);
      bool any = false;
      for (int r = 0; r < R; r++) {
        rows[r] = balanced_split(c->runs_h[r], cs, tv, g);
        any = any || !rows[r].empty();
      }
      if (!any) continue;
      LbPlan p;
      cudaError_t e = full_plan(c, std::vector<int>(R, cs), std::vector<int>(R, tv), best_sv, p);
      p.rows = rows;
      double per = 0.0;
      if (e == cudaSuccess) e = time_plan(c, p, tsteps, e0, e1, &per);
      if (e != cudaSuccess) return bail(e);
      if (per < best_ms) {
        best_ms = per;
        arg = shapes[q].second;
        plan_cs.assign(R, cs);
        plan_tv.assign(R, tv);
        plan_rows = rows;
      }
    }
  }
  // per-run plan
  if (R > 1) {
    std::vector<int> pcs(R, 0), ptv(R, 0);
    std::vector<std::vector<int>> prows(R);
    bool any = false, mixed = false;
    for (int r = 0; r < R; r++) {
      LbPlan p;
      p.cs.assign(R, 0);
      p.tv.assign(R, 0);
      p.active.assign(R, 0);
      p.active[r] = 1;
      p.variant = best_sv;
      cudaError_t e = upload_stream_table(c, std::vector<int>{r});
      p.table = c->d_runs_stream;
      p.nstream = 1;
      for (int q = 0; q < 3; q++) p.tiles[q] = c->stream_tiles[q];
      double run_best = 0.0;
      if (e == cudaSuccess) e = time_plan(c, p, tsteps, e0, e1, &run_best);
      if (e != cudaSuccess) return bail(e);
      p.nstream = 0;
      int ccs = 0, ctv = 0;  // the run's fastest cluster shape, even if streaming beats it
      double cbest = 1e30;
      for (const int cs : kClusterSizes)
        for (int tv = 0; tv < ntv; tv++) {
          if (!shape_fits(c->runs_h[r], cs, tv)) continue;
          p.cs[r] = cs;
          p.tv[r] = tv;
          double per = 0.0;
          if (time_plan(c, p, tsteps, e0, e1, &per) != cudaSuccess) {
            cudaGetLastError();
            continue;
          }
          if (per < cbest) {
            cbest = per;
            ccs = cs;
            ctv = tv;
          }
          if (per < run_best) {
            run_best = per;
            pcs[r] = cs;
            ptv[r] = tv;
          }
        }
      if (ccs > 0) {  // that shape balanced: it may beat streaming where the even split does not
        p.cs[r] = ccs;
        p.tv[r] = ctv;
        p.rows.assign(R, std::vector<int>());
        for (double g : kBalanceGamma) {
          std::vector<int> row0 = balanced_split(c->runs_h[r], ccs, ctv, g);
          if (row0.empty() || row0 == p.rows[r]) continue;
          p.rows[r] = row0;
          double per = 0.0;
          const cudaError_t te = time_plan(c, p, tsteps, e0, e1, &per);
          if (te != cudaSuccess) return bail(te);
          if (per < run_best) {
            run_best = per;
            pcs[r] = ccs;
            ptv[r] = ctv;
            prows[r] = row0;
          }
        }
        if (pcs[r] != ccs || ptv[r] != ctv) prows[r].clear();  // another shape (or streaming) won
      }
      any = any || pcs[r] > 0;
    }
    for (int r = 0; r < R; r++) mixed = mixed || pcs[r] != pcs[0] || ptv[r] != ptv[0];
    if (any && mixed) {
      LbPlan p;
      cudaError_t e = full_plan(c, pcs, ptv, best_sv, p);
      p.rows = prows;
      double per = 0.0;
      if (e == cudaSuccess) e = time_plan(c, p, tsteps, e0, e1, &per);
      if (e != cudaSuccess) return bail(e);
      if (per < best_ms) {
        best_ms = per;
        arg = CLBM_VARIANT_PER_RUN;
        plan_cs = pcs;
        plan_tv = ptv;
        plan_rows = prows;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CK(set_plan(c, plan_cs, plan_tv, best_sv, plan_rows));
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_cache[key] = TuneResult{arg, plan_cs, plan_tv, best_sv, plan_rows};
  }
  if (best) *best = arg;
  return CLBM_OK;
}

extern "C" int clbm_set_step_variant(clbm_ctx *c, int variant) {
  if (!c) return fail(CLBM_ERR_INVALID, "ctx is NULL");
  if (variant < 0 || variant >= variant_count()) return fail(CLBM_ERR_INVALID, "no such variant");
  if (variant >= step_variant_count()) {
    if (c->precision != CLBM_FP32) return fail(CLBM_ERR_INVALID, "cluster-resident intervals are FP32 only");
    int cs, tv;
    variant_shape(variant, cs, tv);
    for (const RunDev &R : c->runs_h)
      if (!shape_fits(R, cs, tv)) return fail(CLBM_ERR_INVALID, "cluster shape does not fit this workload");
  }
  CK(apply_variant(c, variant));
  return CLBM_OK;
}

extern "C" int clbm_set_run_variants(clbm_ctx *c, const int *variants) {
  if (!c || !variants) return fail(CLBM_ERR_INVALID, "NULL argument");
  std::vector<int> cs(c->nruns), tv(c->nruns);
  int sv = -1;
  for (int r = 0; r < c->nruns; r++) {
    const int v = variants[r];
    if (v < 0 || v >= variant_count()) return fail(CLBM_ERR_INVALID, "no such variant");
    variant_shape(v, cs[r], tv[r]);
    if (!cs[r]) {
      if (sv >= 0 && sv != v) return fail(CLBM_ERR_INVALID, "the streaming runs must share one streaming variant");
      sv = v;
    } else {
      if (c->precision != CLBM_FP32) return fail(CLBM_ERR_INVALID, "cluster-resident intervals are FP32 only");
      if (!shape_fits(c->runs_h[r], cs[r], tv[r]))
        return fail(CLBM_ERR_INVALID, "cluster shape does not fit this run's lattice");
    }
  }
  CK(set_plan(c, cs, tv, sv >= 0 ? sv : c->step_variant));
  return CLBM_OK;
}

extern "C" int clbm_band_rows(const clbm_run_desc *run, int cluster_size, double gamma, int *rows) {
  if (!run || !rows) return fail(CLBM_ERR_INVALID, "NULL argument");
  if (cluster_size < 1 || cluster_size > MAX_CLUSTER || cluster_size > run->height)
    return fail(CLBM_ERR_INVALID, "cluster size out of range");
  std::vector<int> row0(cluster_size + 1);
  if (!balanced_band_rows(run->width, run->height, run->xmin, run->xmax, run->ymin, run->ymax, cluster_size,
                          gamma, temporal_rows_limit(run->width), row0.data()))
    return fail(CLBM_ERR_INVALID, "no band split of this lattice fits in shared memory");
  for (int b = 0; b < cluster_size; b++) rows[b] = row0[b + 1] - row0[b];
  return CLBM_OK;
}

extern "C" int clbm_set_band_rows(clbm_ctx *c, int run, const int *rows, int nbands) {
  if (!c || (!rows && nbands)) return fail(CLBM_ERR_INVALID, "NULL argument");
  if (run < 0 || run >= c->nruns) return fail(CLBM_ERR_INVALID, "run out of range");
  const RunDev &R = c->runs_h[run];
  if (nbands == 0) {  // back to the even split
    c->run_rows[run].clear();
    destroy_graphs(c);
    return CLBM_OK;
  }
  if (c->run_cs[run] == 0 || nbands != c->run_cs[run])
    return fail(CLBM_ERR_INVALID, "nbands must equal the run's cluster size (a cluster-resident variant)");
  std::vector<int> row0(nbands + 1, 0);
  for (int b = 0; b < nbands; b++) {
    if (rows[b] < 1) return fail(CLBM_ERR_INVALID, "every band needs at least one row");
    row0[b + 1] = row0[b] + rows[b];
  }
  if (row0[nbands] != R.H) return fail(CLBM_ERR_INVALID, "band rows must sum to the lattice height");
  if (temporal_max_clusters(nbands, c->run_tv[run], R.W, split_rows_max(row0), R.field_mode != 0) < 1)
    return fail(CLBM_ERR_INVALID, "the largest band does not fit in shared memory at this variant");
  c->run_rows[run] = row0;
  destroy_graphs(c);
  return CLBM_OK;
}

extern "C" int clbm_get_band_rows(clbm_ctx *c, int run, int *rows, int *nbands) {
  if (!c || !rows || !nbands) return fail(CLBM_ERR_INVALID, "NULL argument");
  if (run < 0 || run >= c->nruns) return fail(CLBM_ERR_INVALID, "run out of range");
  const int cs = c->run_cs[run];
  *nbands = cs;
  if (!cs) return CLBM_OK;
  std::vector<int> row0 = c->run_rows[run];
  if ((int)row0.size() != cs + 1) {
    row0.assign(cs + 1, 0);
    even_band_rows(c->runs_h[run].H, cs, row0.data());
  }
  for (int b = 0; b < cs; b++) rows[b] = row0[b + 1] - row0[b];
  return CLBM_OK;
}

extern "C" int clbm_get_run_variants(clbm_ctx *c, int *variants) {
  if (!c || !variants) return fail(CLBM_ERR_INVALID, "NULL argument");
  for (int r = 0; r < c->nruns; r++)
    variants[r] = c->run_cs[r] ? variant_index(c->run_cs[r], c->run_tv[r]) : c->step_variant;
  return CLBM_OK;
}

extern "C" int clbm_scgf(clbm_ctx *c, int run, int first, int count, double dT, double *psi) {
  if (int s = check_run(c, run)) return s;
  if (!psi || count < 1 || !(dT > 0.0)) return fail(CLBM_ERR_INVALID, "need count >= 1, dT > 0, psi");
  int done = 0;
  CK(cudaMemcpyAsync(&done, &c->d.state[run].interval, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (first < 0 || first + count > done || first + count > c->d.max_intervals)
    return fail(CLBM_ERR_INVALID, "requested intervals outside the recorded history");
  double *d_out = nullptr;
  CK(cudaMallocAsync((void **)&d_out, sizeof(double), c->stream));
  cudaError_t e = launch_scgf(c->d.logr + (size_t)run * c->d.max_intervals, first, count, dT, d_out, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(psi, d_out, sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  cudaFreeAsync(d_out, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return clbm_status_from_cuda(e);
}

extern "C" int clbm_set_pending_labels(clbm_ctx *c, int run, const int *labels) {
  if (int s = check_run(c, run)) return s;
  if (!labels) return fail(CLBM_ERR_INVALID, "labels is NULL");
  const RunDev &R = c->runs_h[run];
  std::vector<int> mark(R.nclones);
  for (int j = 0; j < R.nclones; j++) {
    if (labels[j] < 0 || labels[j] >= R.nclones) return fail(CLBM_ERR_INVALID, "label out of range");
    mark[j] = labels[j] != j;
    if (mark[j] && labels[labels[j]] != labels[j]) return fail(CLBM_ERR_INVALID, "a parent is itself a copy");
  }
  c->pending = true;
  CK(cudaMemcpyAsync(c->d.labels + R.clone_base, labels, sizeof(int) * R.nclones, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->d.mark + R.clone_base, mark.data(), sizeof(int) * R.nclones, cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return CLBM_OK;
}

// ---------------------------------------------------------------------------
// Adjoint of the interval-integrated drag (kernels in clbm_adjoint.cu).
static cudaError_t adj_reserve(char *&p, size_t &have, size_t need) {
  if (have >= need && p) return cudaSuccess;
  if (p) cudaFree(p);
  p = nullptr;
  have = 0;
  cudaError_t e = cudaMalloc((void **)&p, need);
  if (e == cudaSuccess) have = need;
  return e;
}

extern "C" int clbm_drag_fwd(clbm_ctx *c, int steps, int every, double *J) {
  if (!c) return fail(CLBM_ERR_INVALID, "ctx is NULL");
  if (steps < 1 || steps > c->max_steps || every < 1) return fail(CLBM_ERR_INVALID, "bad steps / checkpoint period");
  if (c->pending) return fail(CLBM_ERR_INVALID, "a clone step is pending; run an interval first");
  const bool f64 = c->precision == CLBM_FP64;
  const size_t pop = c->pop_elems * c->elem_size;
  const size_t nckpt = (size_t)(steps + every - 1) / every;
  size_t have_s0 = c->adj.s0 ? pop : 0, have_ck = c->adj.nckpt * pop, have_seg = c->adj.nseg * pop;
  size_t have_sig0 = c->adj.sig[0] ? pop : 0, have_sig1 = c->adj.sig[1] ? pop : 0;
  CK(adj_reserve(c->adj.s0, have_s0, pop));
  CK(adj_reserve(c->adj.ckpt, have_ck, nckpt * pop));
  c->adj.nckpt = have_ck / pop;
  CK(adj_reserve(c->adj.seg, have_seg, (size_t)every * pop));
  c->adj.nseg = have_seg / pop;
  CK(adj_reserve(c->adj.sig[0], have_sig0, pop));
  CK(adj_reserve(c->adj.sig[1], have_sig1, pop));
  cudaStream_t s = c->stream;
  CK(cudaMemcpyAsync(c->adj.s0, c->pop[c->s_buf], pop, cudaMemcpyDeviceToDevice, s));
  auto loc = [&](int t) -> char * {
    return (t % every == 0) ? c->adj.ckpt + (size_t)(t / every) * pop : c->adj.sig[t % 2];
  };
  // runs with a random body-force field step under the fields of the last
  // interval (the ones clbm_get_field_map returns)
  ReseedArgs ra{c->d.runs, c->nruns, c->adj.s0, loc(0), c->d_identity, c->d_zeros, c->d.pert,
                c->d.prefactors, c->d.snaps, c->d.state, c->d.err, c->d_maps};
  CK(launch_reseed(f64, ra, c->total_blocks, s));
  for (int t = 0; t < steps; t++) {
    char *dst = (t + 1 < steps) ? loc(t + 1) : c->adj.sig[(t + 1) % 2];
    StepArgs a{c->d.runs, c->nruns, t, loc(t), dst, c->d.terms, c->d.term_slab, c->d.err,
               c->total_clones, c->max_nodes, {c->total_tiles[0], c->total_tiles[1], c->total_tiles[2]},
               c->d_maps};
    CK(launch_step(f64, false, a, c->total_blocks, s, c->step_variant));
  }
  CK(launch_drag_reduce(f64, c->d, c->nruns, c->total_clones, steps, c->any_stress, c->any_momentum, s));
  if (J) CK(cudaMemcpyAsync(J, c->d.sacc, sizeof(double) * c->total_clones, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  c->adj.steps = steps;
  c->adj.every = every;
  c->adj.result = -1;
  c->last_steps = steps;  // clbm_get_drag returns this forward's drag series
  return check_error_word(c);
}

extern "C" int clbm_drag_bwd(clbm_ctx *c) {
  if (!c) return fail(CLBM_ERR_INVALID, "ctx is NULL");
  if (c->adj.steps < 1) return fail(CLBM_ERR_INVALID, "clbm_drag_bwd before clbm_drag_fwd");
  const bool f64 = c->precision == CLBM_FP64;
  const size_t pop = c->pop_elems * c->elem_size;
  const int T = c->adj.steps, C = c->adj.every;
  cudaStream_t s = c->stream;
  const int nseg = (T + C - 1) / C;
  int cur = 0;  // sig[cur] holds sigma_{t+1}
  auto segP = [&](int lo, int p) -> char * {
    return p == lo ? c->adj.ckpt + (size_t)(lo / C) * pop : c->adj.seg + (size_t)(p - lo) * pop;
  };
  for (int k = nseg - 1; k >= 0; k--) {
    const int lo = k * C, hi = std::min(lo + C, T) - 1;
    for (int p = lo; p < hi; p++) {  // recompute P_lo .. P_hi from the checkpoint (step p of the forward)
      StepArgs a{c->d.runs, c->nruns, p, segP(lo, p), segP(lo, p + 1), c->d.terms, c->d.term_slab,
                 c->d.err, c->total_clones, c->max_nodes,
                 {c->total_tiles[0], c->total_tiles[1], c->total_tiles[2]}, c->d_maps};
      CK(launch_step(f64, false, a, c->total_blocks, s, c->step_variant));
    }
    for (int p = hi; p >= lo; p--) {
      if (p == T - 1) {
        CK(launch_adj_init(f64, c->d.runs, c->nruns, segP(lo, p), c->adj.sig[cur], c->total_blocks, s));
      } else {
        CK(launch_adj_step(f64, c->d.runs, c->nruns, c->adj.sig[cur], c->adj.sig[1 - cur], segP(lo, p),
                           true, false, p + 1, c->d_maps, c->total_blocks, s));
        cur = 1 - cur;
      }
    }
  }
  CK(launch_adj_step(f64, c->d.runs, c->nruns, c->adj.sig[cur], c->adj.sig[1 - cur], c->adj.s0, false,
                     true, 0, c->d_maps, c->total_blocks, s));
  c->adj.result = 1 - cur;
  CK(cudaStreamSynchronize(s));
  return check_error_word(c);
}

extern "C" int clbm_get_drag_grad_aos_f64(clbm_ctx *c, int run, int clone, double *aos) {
  if (int st = check_run(c, run)) return st;
  const RunDev &R = c->runs_h[run];
  if (clone < 0 || clone >= R.nclones || !aos) return fail(CLBM_ERR_INVALID, "bad clone or NULL array");
  if (c->adj.result < 0) return fail(CLBM_ERR_INVALID, "no gradient: call clbm_drag_bwd first");
  const size_t n = 9 * (size_t)R.nodes;
  double *stage = nullptr;
  CK(cudaMallocAsync((void **)&stage, n * 8, c->stream));
  cudaError_t e = launch_soa_to_aos(c->precision == CLBM_FP64, c->d.runs, run, R.nodes, clone,
                                    c->adj.sig[c->adj.result], stage, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(aos, stage, n * 8, cudaMemcpyDeviceToHost, c->stream);
  cudaFreeAsync(stage, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return clbm_status_from_cuda(e);
  if (c->precision != CLBM_FP64)  // soa_to_aos adds back w[k] for states; a gradient has no shift
    for (size_t i = 0; i < n; i++) aos[i] -= w_of((int)(i % 9));
  return CLBM_OK;
}

// ---------------------------------------------------------------------------
// Lineage reconstruction (post_processing/reconstruction.cpp:35-109 on the
// device): keep every interval's drag series and labels, then trace each
// final slot back through its ancestors.
extern "C" int clbm_enable_history(clbm_ctx *c, int max_intervals) {
  if (!c) return fail(CLBM_ERR_INVALID, "ctx is NULL");
  if (max_intervals < 1 || max_intervals > c->d.max_intervals) return fail(CLBM_ERR_INVALID, "max_intervals out of range");
  if (c->hist_drag) cudaFree(c->hist_drag);
  if (c->hist_labels) cudaFree(c->hist_labels);
  c->hist_drag = nullptr;
  c->hist_labels = nullptr;
  c->hist_max = 0;
  CK(cudaMalloc((void **)&c->hist_drag, sizeof(double) * (size_t)max_intervals * c->total_clones * c->max_steps));
  CK(cudaMalloc((void **)&c->hist_labels, sizeof(int) * (size_t)max_intervals * c->total_clones));
  c->hist_max = max_intervals;
  c->hist_steps = 0;
  c->hist_steps_varied = false;
  destroy_graphs(c);
  int done = 0;
  CK(cudaMemcpyAsync(&done, &c->d.state[0].interval, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (done != 0) return fail(CLBM_ERR_INVALID, "enable the history before the first interval");
  return CLBM_OK;
}

extern "C" int clbm_reconstruct_lineages(clbm_ctx *c, int run, int *nintervals, double *out,
                                         int *ancestors) {
  if (int st = check_run(c, run)) return st;
  if (c->hist_max < 1) return fail(CLBM_ERR_INVALID, "history not enabled (clbm_enable_history)");
  if (c->hist_steps_varied) return fail(CLBM_ERR_INVALID, "intervals of different lengths in the history");
  int done = 0;
  CK(cudaMemcpyAsync(&done, &c->d.state[0].interval, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  const int n = std::min(done, c->hist_max);
  if (nintervals) *nintervals = n;
  if (n < 1 || (!out && !ancestors)) return CLBM_OK;
  const RunDev &R = c->runs_h[run];
  const int steps = c->hist_steps;
  int *d_anc = nullptr;
  double *d_out = nullptr;
  CK(cudaMallocAsync((void **)&d_anc, sizeof(int) * (size_t)R.nclones * n, c->stream));
  cudaError_t e = cudaMallocAsync((void **)&d_out, sizeof(double) * (size_t)R.nclones * n * steps, c->stream);
  if (e == cudaSuccess)
    e = launch_reconstruct(c->hist_drag, c->hist_labels, c->total_clones, R.clone_base, R.nclones, n, steps,
                           c->max_steps, d_anc, d_out, c->stream);
  if (e == cudaSuccess && out)
    e = cudaMemcpyAsync(out, d_out, sizeof(double) * (size_t)R.nclones * n * steps, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess && ancestors)
    e = cudaMemcpyAsync(ancestors, d_anc, sizeof(int) * (size_t)R.nclones * n, cudaMemcpyDeviceToHost, c->stream);
  cudaFreeAsync(d_anc, c->stream);
  if (d_out) cudaFreeAsync(d_out, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return clbm_status_from_cuda(e);
}

extern "C" int clbm_macro_fields(clbm_ctx *c, int run, int clone, double *rho, double *ux, double *uy) {
  if (int st = check_run(c, run)) return st;
  const RunDev &R = c->runs_h[run];
  if (clone < 0 || clone >= R.nclones || !rho || !ux || !uy) return fail(CLBM_ERR_INVALID, "bad clone or NULL array");
  if (c->pending) return fail(CLBM_ERR_INVALID, "a clone step is pending; run an interval first");
  const size_t n = R.nodes;
  double *d = nullptr;
  CK(cudaMallocAsync((void **)&d, 3 * n * sizeof(double), c->stream));
  cudaError_t e = launch_macro(c->precision == CLBM_FP64, c->d.runs, run, clone, R.nodes, c->pop[c->s_buf], d,
                               d + n, d + 2 * n, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(rho, d, n * 8, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(ux, d + n, n * 8, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(uy, d + 2 * n, n * 8, cudaMemcpyDeviceToHost, c->stream);
  cudaFreeAsync(d, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return clbm_status_from_cuda(e);
}

extern "C" int clbm_get_field_map(clbm_ctx *c, int run, int clone, double *map, int *negative) {
  if (int st = check_run(c, run)) return st;
  const RunDev &R = c->runs_h[run];
  if (!R.field_mode) return fail(CLBM_ERR_INVALID, "run has no random field");
  if (clone < 0 || clone >= R.nclones) return fail(CLBM_ERR_INVALID, "bad clone");
  if (negative) *negative = c->field_negative[run];
  if (!map) return CLBM_OK;
  std::vector<float> f(R.nodes);
  CK(cudaMemcpyAsync(f.data(), c->d_maps + R.map_base + (size_t)clone * R.nodes, sizeof(float) * R.nodes,
                     cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int x = 0; x < R.W; x++)
    for (int y = 0; y < R.H; y++) map[y + (size_t)R.H * x] = (double)f[(size_t)y * R.W + x];
  return CLBM_OK;
}

extern "C" int clbm_ref_random_field(int dx, int dy, double sigma, unsigned long long seed, int draw,
                                     double *map, int *negative) {
  if (dx < 3 || dy < 4 || dx > 1024 || dy > 1024 || !(sigma > 0) || draw < 0 || !map)
    return fail(CLBM_ERR_INVALID, "clbm_ref_random_field: need 3 <= dx <= 1024, 4 <= dy <= 1024, sigma > 0, "
                                  "draw >= 0, map != NULL");
  // a one-clone context whose only use is its field tables and kernels (the
  // square is a placeholder: nothing is stepped)
  clbm_run_desc d{};
  d.width = dx;
  d.height = dy;
  d.xmin = 0;
  d.xmax = 1;
  d.ymin = 1;
  d.ymax = 2;
  d.nclones = 1;
  d.ranks = 1;
  d.tau = 1.0;
  d.dt = 1.0;
  d.force_scale = 1.0;
  d.seed = seed;
  d.field_mode = 1;
  d.field_steps = 1;
  d.field_eps = 1.0;
  d.field_sigma = sigma;
  clbm_ctx *c = nullptr;
  if (int st = clbm_create(&d, 1, CLBM_FP32, 1, 0, &c)) return st;
  cudaError_t e = cudaMemcpyAsync((char *)c->d.state + offsetof(RunState, interval), &draw, sizeof(int),
                                  cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) {
    FieldArgs fa{c->d.runs, c->nruns, c->d.state, c->d_spec, c->d_tw, c->d_ybuf, c->d_maps, c->d_fa, c->d.err, c->d_flist};
    e = launch_fields(fa, c->total_clones, c->field_max_w, c->field_max_m1, c->field_max_m2,
                      c->field_max_tiles2, c->stream);
  }
  int st = clbm_status_from_cuda(e);
  if (st == CLBM_OK) st = clbm_get_field_map(c, 0, 0, map, negative);
  clbm_destroy(c);
  return st;
}
