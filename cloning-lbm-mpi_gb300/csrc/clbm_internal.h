// clbm_internal.h -- structures shared by the kernel translation units and the
// host-side context (clbm_api.cu).  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>

#include "clbm_common.cuh"

namespace clbm {

constexpr int MAX_RANKS = 64;   // virtual MPI ranks per run
constexpr int MAX_SNAP = 64;    // perturbation snapshots per run
constexpr int STEP_BLOCK = 256; // nodes per block of the step kernels

// Per-run state that lives on the device between kernels (random-stream
// positions, interval counter), so that captured CUDA graphs replay with the
// state advancing on the device.
struct RunState {
  unsigned long long d48[MAX_RANKS];  // drand48 X of each virtual rank
  GlibcRand rnd;                      // rank 0's glibc rand() state
  int interval;                       // cloning intervals completed
  int ncomm;                          // clone copies of the last clone step
  int ncopies_drawn;                  // NcPrime of the last clone step
  int pad_;
  double rbar;                        // R_t of the last clone step
  double logr;                        // log R_t (finite where R_t overflows)
};

// Device arrays of one context (all indexed by global clone index unless
// stated otherwise).
struct DevArrays {
  RunDev *runs;       // [nruns]
  RunState *state;    // [nruns]
  double *sacc;       // weight integral s_j = dt * sum F of the last interval
  double *drag;       // per run: [nclones][max_steps] F values, run base = clone_base*max_steps
  double *weights;    // exp(alpha s_j) (reference) / exp(alpha s_j) (systematic)
  int *labels;        // parent slot (run-local) of each slot, pending until the next interval
  int *mark;          // 1 = slot receives a copy and is perturbed at the next interval
  int *copies_pre;    // copy numbers drawn
  int *copies_post;   // after the kill/duplicate correction
  double *prefactors; // [clone][MAX_SNAP] snapshot-mix prefactors of marked clones
  double *pert;       // [clone][2] (weight, 1/a) of the snapshot mix
  double *partials;   // [clone][blocks_per_clone][2] norm partial sums
  int *scratch_i;     // per run: 4*nclones+4 ints (copy numbers, sampling array, extras)
  double *scratch_d;  // per run: nclones doubles (prefix sums)
  double *snaps;      // per run: nsnap * 9 * plane FP64, SoA like the populations
  double *rvalues;    // per run: [max_intervals] R_t history
  double *logr;       // per run: [max_intervals] log R_t history
  unsigned *err;      // device error word
  void *terms;        // [max_steps][slab] drag terms (double or float)
  long long term_slab;// terms per step over all runs
  int max_steps;
  int max_intervals;
};

struct FieldArgs {
  const RunDev *runs;
  int nruns;
  const RunState *state;   // interval counter (random-stream counter)
  const float *spec;       // sqrt spectra, [M1][M2] per field run
  const float2 *twiddles;  // exp(-2 pi i k / M1), exp(-2 pi i k / M2) per field run
  float2 *ybuf;            // stage-1 results: [2][W][M2] floats per clone (real, imaginary planes)
  float *maps;             // fields, W*H per clone, node order y*W + x
  const float *dft;        // stage-1 DFT operand images (tensor-core layout), per field run
  unsigned *err;           // device error word
  const int *flist;        // kept embedding rows a and columns b, per field run
};

struct StepArgs {
  const RunDev *runs;
  int nruns;
  int step;           // step index within the interval (drag-term slab)
  const void *src;    // post-collision populations of the previous step
  void *dst;          // this step's post-collision (or, on the last step, pre-collision) populations
  void *terms;        // base of the term slabs
  long long term_slab;
  unsigned *err;
  int total_clones;
  int max_nodes;
  int total_tiles[3]; // FP32 step grid for tiles of 128 / 256 / 512 nodes
  const float *maps;  // random body-force fields (nullable)
};

struct ReseedArgs {
  const RunDev *runs;
  int nruns;
  const void *src;    // pre-collision state S of every slot's parent
  void *dst;          // post-collision populations P of the next interval's first step
  const int *labels;
  const int *mark;
  const double *pert;       // (weight, 1/a) per clone
  const double *prefactors; // [clone][MAX_SNAP]
  const double *snaps;
  const RunState *state;    // interval counter
  unsigned *err;
  const float *maps;        // random body-force fields (nullable)
};

// largest cluster of the cluster-resident interval kernel (non-portable size)
constexpr int MAX_CLUSTER = 16;

struct TemporalArgs {
  RunDev rd;          // the run, by value: kernel-parameter space, never aliased
  int run;
  int steps;
  const float *src;   // P_0 (post-collision) of every clone of the run
  float *dst;         // S_T (pre-collision) after the interval
  float *terms;       // base of the drag-term slabs
  long long term_slab;
  unsigned *err;
  const float *maps;  // random body-force fields (nullable)
  // band b of a clone (CTA of cluster rank b) holds the lattice rows
  // [band_row0[b], band_row0[b + 1]); band_row0[cs] = H
  int band_row0[MAX_CLUSTER + 1];
  // fused: the kernel forms P_0 itself from the previous interval's S in
  // rs.src (parent copy, perturbation, first collision: the reseed of every
  // node, clbm_step.cu), instead of reading it from src
  int fused;
  ReseedArgs rs;
};


// kernel launchers (clbm_step.cu, clbm_cloning.cu)
cudaError_t launch_step(bool f64, bool last, const StepArgs &a, int blocks, cudaStream_t s,
                        int variant);
int step_variant_count();
int step_variant_block(int variant);
cudaError_t launch_reseed(bool f64, const ReseedArgs &a, int blocks, cudaStream_t s);
cudaError_t launch_perturb_norms(bool f64, const RunDev *runs, int nruns, const void *src,
                                 const int *labels, const int *mark, const double *prefactors,
                                 const double *snaps, double *partials, double *pert,
                                 int blocks, int total_clones, cudaStream_t s);
cudaError_t launch_drag_reduce(bool f64, const DevArrays &d, int nruns, int total_clones,
                               int steps, bool stress, bool momentum, cudaStream_t s);
cudaError_t launch_clone(const DevArrays &d, int nruns, cudaStream_t s);
cudaError_t launch_adj_init(bool f64, const RunDev *runs, int nruns, const void *P, void *sigma,
                            int blocks, cudaStream_t s);
cudaError_t launch_adj_step(bool f64, const RunDev *runs, int nruns, const void *sigma_in,
                            void *sigma_out, const void *P, bool with_drag, bool from_s0, int t,
                            const float *maps, int blocks, cudaStream_t s);
cudaError_t launch_hist_drag(const DevArrays &d, int total_clones, int steps, double *hist, int max_hist,
                             cudaStream_t s);
cudaError_t launch_hist_labels(const DevArrays &d, int total_clones, int *hist, int max_hist,
                               cudaStream_t s);
cudaError_t launch_reconstruct(const double *hist_drag, const int *hist_labels, int total_clones,
                               int clone_base, int nclones, int n, int steps, int max_steps,
                               int *anc, double *out, cudaStream_t s);
cudaError_t launch_fields(const FieldArgs &a, int total_clones, int max_w, int max_m1, int max_m2,
                          int max_tiles2, cudaStream_t s);
// rows of the tensor-core stage-1 operand (2W rounded up to the 128-row tile)
// and its 32-wide K chunks (twice the kept rows a, rounded up); the image holds
// mpad * 32 * kchunks floats
inline int field_dft_mpad(int W) { return (2 * W + 127) / 128 * 128; }
inline int field_dft_kchunks(int na) { return (2 * na + 31) / 32; }
// row pitch (floats) of the stage-1 output Y of nb kept columns: a multiple of
// 4, so a row starts on a 16-byte boundary and the stores are 16-byte vectors
__host__ __device__ inline int field_y_pitch(int nb) { return (nb + 3) & ~3; }
void build_field_dft_image(int W, int M1, const int *alist, int na, int mpad, int kchunks, float *out);
// cluster-resident interval kernel (clbm_temporal.cu): launch with the bands
// of a.band_row0; resident clusters of a shape whose largest band has
// rows_max rows (0: it cannot run); the most rows a band of width W can hold
cudaError_t launch_temporal(const TemporalArgs &a, int cs, int variant, int nclones, int W,
                            cudaStream_t s);
int temporal_max_clusters(int cs, int variant, int W, int rows_max, bool field);
int temporal_rows_limit(int W);
int temporal_variant_count();
// band splits (clbm_bands.cu): row0[0..cs] of H rows in cs bands, the first
// H % cs one row more; or balanced for an estimated per-step cost in which a
// node on the general path (the square's box) counts 1 + gamma and a node of
// a wall or band-edge row 1 + gamma / 4 (false: no split within the row limit)
void even_band_rows(int H, int cs, int *row0);
bool balanced_band_rows(int W, int H, int xmin, int xmax, int ymin, int ymax, int cs, double gamma,
                        int rows_limit, int *row0);
cudaError_t launch_scgf(const double *logr, int first, int count, double dT, double *out,
                        cudaStream_t s);
cudaError_t launch_init_equilibrium(bool f64, const RunDev *runs, int nruns, int run, void *pop,
                                    double u0, double noise, unsigned long long seed, int blocks,
                                    cudaStream_t s);
cudaError_t launch_aos_to_soa(bool f64, const RunDev *runs, int run, int nodes, int clone0, int nclone,
                              const double *aos, void *pop, cudaStream_t s);
cudaError_t launch_soa_to_aos(bool f64, const RunDev *runs, int run, int nodes, int clone, const void *pop,
                              double *aos, cudaStream_t s);
cudaError_t launch_macro(bool f64, const RunDev *runs, int run, int clone, int nodes, const void *pop,
                         double *rho, double *ux, double *uy, cudaStream_t s);
cudaError_t launch_snaps_to_soa(const RunDev *runs, int run, int nodes, int nsnap, const double *aos,
                                double *snaps, cudaStream_t s);

}  // namespace clbm
