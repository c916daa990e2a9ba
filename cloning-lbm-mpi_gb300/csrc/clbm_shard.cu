// clbm_shard.cu -- host-side plan of the clone exchange when the clones of a
// run are split over several processes (one GPU each).
//
// The reference splits Nc clones over p MPI ranks in contiguous blocks of
// local_Nc = Nc / p and, after the cloning step, walks the copy table
// (clone_to_move, clone_to_erase): sender = ctm / local_Nc, dest =
// cte / local_Nc, a memcpy when both are the same rank, else a blocking
// MPI_Send / MPI_Recv of the N populations with tag = table index
// (src/mpi_LBM_GK_pops_perturb.cpp:650-699).  Here the table is the sampler's
// labels array (slot j takes the state of slot labels[j]; labels[j] == j
// keeps it) and the plan gives each shard its part, every list in ascending
// destination slot so that both ends of a transfer agree on the order.  No
// device is needed: the plan is pure host code, and the transfers are the
// caller's (NCCL send/recv between GPUs, or any transport).
#include <vector>

#include "clbm.h"

extern "C" void clbm_set_error(const char *msg);

extern "C" int clbm_shard_plan(const int *labels, int nclones, int nshards, int shard, clbm_copy *sends,
                               int *nsends, clbm_copy *recvs, int *nrecvs, clbm_copy *locals, int *nlocals) {
  if (!labels || nclones < 1 || nshards < 1 || shard < 0 || shard >= nshards) {
    clbm_set_error("clbm_shard_plan: bad labels, nclones, nshards or shard");
    return CLBM_ERR_INVALID;
  }
  if (nclones % nshards) {
    clbm_set_error("clbm_shard_plan: nclones must be a multiple of nshards (contiguous blocks)");
    return CLBM_ERR_INVALID;
  }
  const int local = nclones / nshards;
  // a parent must keep its own state: every source slot maps to itself
  for (int j = 0; j < nclones; j++) {
    const int p = labels[j];
    if (p < 0 || p >= nclones || labels[p] != p) {
      clbm_set_error("clbm_shard_plan: labels[j] must be a slot that keeps its own state");
      return CLBM_ERR_INVALID;
    }
  }
  int ns = 0, nr = 0, nl = 0;
  for (int j = 0; j < nclones; j++) {
    const int p = labels[j];
    if (p == j) continue;
    const int src = p / local, dst = j / local;
    if (src == shard && dst == shard) {
      if (locals) locals[nl] = clbm_copy{p, j, shard};
      nl++;
    } else if (src == shard) {
      if (sends) sends[ns] = clbm_copy{p, j, dst};
      ns++;
    } else if (dst == shard) {
      if (recvs) recvs[nr] = clbm_copy{p, j, src};
      nr++;
    }
  }
  if (nsends) *nsends = ns;
  if (nrecvs) *nrecvs = nr;
  if (nlocals) *nlocals = nl;
  return CLBM_OK;
}
