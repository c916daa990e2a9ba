// clbm_reseed.cuh -- the first collision of an interval, per node: shared by
// the reseed kernel (clbm_step.cu) and the cluster-resident interval kernel,
// which forms it while loading a clone (clbm_temporal.cu).
#pragma once

#include <cstdint>
#include <type_traits>

#include "clbm_internal.h"
#include "clbm_physics.cuh"

namespace clbm {

template <bool F64>
using pop_t = typename std::conditional<F64, double, float>::type;

// map: the node's random-field value when the collision is under the
// spatial force, beta(x,y) = (1 + eps*map)*beta0 (streamCollCompute.cpp:63)
template <bool F64>
__device__ __forceinline__ void collide_node(const RunDev &R, const pop_t<F64> S[9],
                                             pop_t<F64> P[9], const float *map = nullptr) {
  if constexpr (F64) {
    if (map) {
      const double beta = DMUL(DADD(1.0, DMUL(R.field_eps, (double)*map)), R.beta);
      double wcb[9];
#pragma unroll
      for (int k = 0; k < 9; k++) wcb[k] = DMUL(DMUL(w_of(k), R.cforce), beta);
      collide_ref64(S, P, beta, wcb, R.omega, R.om1);
    } else {
      collide_ref64(S, P, R.beta, R.wcb, R.omega, R.om1);
    }
  } else {
    collide_f32_run(R, S, P, map, R.f_field_eps);
  }
}

__device__ __forceinline__ const float *node_map(const float *maps, const RunDev &R, int clone, int n,
                                                 bool on) {
  return (on && maps) ? maps + R.map_base + (long long)clone * R.nodes + n : nullptr;
}

// Index of population k of node (x,y) in the reference's AoS layout (the
// counter of the node's perturbation draw).
__device__ __forceinline__ uint32_t aos_index(const RunDev &R, int x, int y, int k) {
  return (uint32_t)(k + 9 * (y + R.H * x));
}

// The reseed of fluid node (x,y) (n = y*W + x) of clone `clone` of run R
// (index `run`): the parent slot's state S(labels[j]) (the clone copy, pops
// driver :658-701), perturbed when the slot is a new clone (:412-416: the
// snapshot mix, generatePerturbedState.cpp:4-38, or the counter-based uniform
// noise), collided into P.
template <bool F64>
__device__ __forceinline__ void reseed_node(const ReseedArgs &a, const RunDev &R, int run, int clone, int x, int y,
                                            int n, pop_t<F64> P[9]) {
  using T = pop_t<F64>;
  const int gclone = R.clone_base + clone;
  int parent = a.labels[gclone];
  if (parent < 0 || parent >= R.nclones) {
    atomicOr(a.err, (unsigned)ERR_BAD_PARENT);
    parent = clone;
  }
  const long long plane = R.plane;
  const T *src = (const T *)a.src + R.pop_base + (long long)parent * 9 * plane;
  T S[9];
#pragma unroll
  for (int k = 0; k < 9; k++) S[k] = src[k * plane + n];
  if (R.perturb_mode != 0 && a.mark[gclone]) {
    const int interval = a.state[run].interval;
    const double *pre = a.prefactors + (long long)gclone * MAX_SNAP;
    const double wgt = a.pert[2 * gclone], inv_a = a.pert[2 * gclone + 1];
#pragma unroll
    for (int k = 0; k < 9; k++) {
      double f = F64 ? (double)S[k] : w_of(k) + (double)S[k];
      if (R.perturb_mode == 2) {
        const double u = philox_uniform(R.seed, aos_index(R, x, y, k), (uint32_t)clone,
                                        (uint32_t)interval, (R.run_id << 4) | DOM_PERTURB);
        f = DMUL(f, DADD(1.0, DMUL(R.eps, DSUB(DMUL(2.0, u), 1.0))));
      } else {
        // S = sum_q r_q snap_q in snapshot order; f <- (f + eps*S*weight) / a
        const double *sp = a.snaps + R.snap_base + (long long)k * plane + n;
        double mix = DMUL(pre[0], sp[0]);
        for (int q = 1; q < R.nsnap; q++) mix = DADD(mix, DMUL(pre[q], sp[(long long)q * 9 * plane]));
        f = DMUL(DADD(f, DMUL(DMUL(R.eps, mix), wgt)), inv_a);
      }
      S[k] = F64 ? (T)f : (T)(f - w_of(k));
    }
  }
  collide_node<F64>(R, S, P, node_map(a.maps, R, clone, n, R.field_mode && R.field_steps > 0));
}

}  // namespace clbm
