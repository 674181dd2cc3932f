// float instantiation of the cluster-persistent dGN engine.
#include "dgn_engine.cuh"

namespace tfx {
int launch_dgn_f32(int TS, const tfx_dgn_problem* d_probs, int nprob, const tfx_dgn_options* op, int cluster,
                  const SmemPlan& sp, cudaStream_t st) {
  if (TS == 1) return launch_dgn<float, 1>(d_probs, nprob, op, cluster, sp, st);
  if (TS == 2) return launch_dgn<float, 2>(d_probs, nprob, op, cluster, sp, st);
  return launch_dgn<float, 4>(d_probs, nprob, op, cluster, sp, st);
}
}  // namespace tfx
