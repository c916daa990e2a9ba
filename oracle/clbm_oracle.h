/*
 * clbm_oracle.h -- CPU restatement of the reference cloning-LBM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests/, the smoke
 * entry point and bench.py's CPU-baseline leg may load it; the product library
 * (libclbm) never links or calls it.
 *
 * Every routine is FP64, uses the reference's array-of-structures layout
 * IDX(x,y,k) = k + 9*(y + Dy*x) (src/lbm_src/global.h:4) and evaluates each
 * expression in the reference's operation order, so that, compiled with
 * -ffp-contract=off, it is bit-identical to the reference objects.
 * Geometry is passed explicitly instead of through the reference's globals
 * Dx, Dy, xmin, xmax, ymin, ymax (src/lbm_src/global.h:11-13).
 */
#ifndef CLBM_ORACLE_H
#define CLBM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int nx, ny;                 /* Dx, Dy */
  int xmin, xmax, ymin, ymax; /* square, perimeter nodes inclusive */
} orc_geom;

/* ---- LBM core (src/lbm_src/*.cpp) ---------------------------------------- */
void orc_stream_collide(const orc_geom *g, double *fin, double *fout,
                        double *rho, double *ux, double *uy, double beta,
                        double tau);
void orc_stream_collide_spatial(const orc_geom *g, double *fin, double *fout,
                                double *rho, double *ux, double *uy,
                                double beta0, const double *map, double tau,
                                double eps);
void orc_walls_bb(const orc_geom *g, double *fout, const double *fin);
void orc_square_bb(const orc_geom *g, double *fout, const double *fin);
void orc_interior_reset(const orc_geom *g, double *fout);
double orc_force_on_square(const orc_geom *g, const double *f, double omega);
/* momentum-exchange x-drag on the square of a streamed, bounced state f:
 * per perimeter node sum_k -2 c_kx f_k over the slots the square bounces
 * back, nodes in the West, East, North, South order of the stress
 * integration (corners in West / East), summed as 32 strided lane partials
 * followed by an xor butterfly (the libclbm momentum-exchange reduction). */
double orc_force_momentum_exchange(const orc_geom *g, const double *f);
/* one full LB step as the drivers chain it; *state and *scratch are swapped */
void orc_lbm_step(const orc_geom *g, double **state, double **scratch,
                  double *rho, double *ux, double *uy, double beta,
                  const double *map, double tau, double eps);
/* which of the 9 outgoing slots of node (x,y) the reference overwrites by
 * bounce-back (bit k set => fout(x,y,k) = post-collision fin(x,y,opp[k])),
 * bit 9 set => node is inside the square (reset to w[k]). */
int orc_bounce_mask(const orc_geom *g, int x, int y);

/* ---- random streams -------------------------------------------------------- */
typedef struct { uint64_t x; } orc_drand48;           /* POSIX drand48 LCG */
void orc_drand48_init_default(orc_drand48 *s);
double orc_drand48_next(orc_drand48 *s);
void orc_drand48_skip(orc_drand48 *s, uint64_t n);
typedef struct { uint32_t r[34]; int i; } orc_glibc_rand;  /* glibc rand() */
void orc_glibc_srand(orc_glibc_rand *s, uint32_t seed);
int32_t orc_glibc_rand_next(orc_glibc_rand *s);
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]);
double orc_philox_uniform(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2,
                          uint32_t c3);

/* ---- perturbation (src/perturbation_routines/generatePerturbedState.cpp) --- */
void orc_perturb_mix(double *fin, const double *snaps, int nsnap, int n,
                     double eps, const double *prefactors);
void orc_perturb_uniform(double *fin, const orc_geom *g, double eps,
                         uint64_t seed, uint32_t run, uint32_t clone,
                         uint32_t interval);
void orc_init_equilibrium(double *fin, const orc_geom *g, double u0,
                          double noise, uint64_t seed, uint32_t run,
                          uint32_t clone);

/* ---- cloning step (src/mpi_LBM_GK_pops_perturb.cpp:487-624) ------------------ */
typedef struct {
  double rbar;      /* R_t, the normalised mean weight */
  double logr;      /* log R_t (finite where R_t itself overflows) */
  int ncopies_drawn;/* NcPrime */
  int ncomm;        /* number of clone copies */
  int status;       /* 0 ok, <0 error */
} orc_clone_result;
orc_clone_result orc_clone_reference(int nc, int ranks, const double *s,
                                     orc_drand48 *master, orc_glibc_rand *rnd,
                                     int *copies_pre, int *copies_post,
                                     int *labels, int *table);
orc_clone_result orc_clone_systematic(int nc, const double *logw, double u,
                                      int *copies, int *labels, int *table);

/* ---- whole sampler ----------------------------------------------------------- */
enum { ORC_PERTURB_NONE = 0, ORC_PERTURB_MIX = 1, ORC_PERTURB_UNIFORM = 2 };
enum { ORC_RESAMPLE_REFERENCE = 0, ORC_RESAMPLE_SYSTEMATIC = 1 };
typedef struct {
  orc_geom g;
  int nclones, steps, intervals, ranks;
  double tau, beta, alpha, force_scale, force_shift, dt;
  int perturb_mode, resample_mode, nsnap;
  double eps;
  uint64_t seed;
  uint32_t run;
  int drag_mode; /* 0 stress integration (the reference), 1 momentum exchange */
} orc_sampler_cfg;
int orc_run_sampler(const orc_sampler_cfg *cfg, double *states,
                    const double *snaps, double *drag, int *labels,
                    double *rvalues, double *logr, double *weights,
                    int *copies);

/* ---- CPU baseline timing: nclones independent clones, nthreads threads ---- */
double orc_bench_lbm(const orc_geom *g, int nclones, int steps, double tau,
                     double beta, int nthreads, double *checksum);

#ifdef __cplusplus
}
#endif
#endif
