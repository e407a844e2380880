// Pair stage with a Kahan-compensated reduction over the scatter points
// (sss_tof_problem.flags & SSS_FLAG_KAHAN).  Each lane sums one scatter
// point's voxels in registers as usual, then adds that partial into its
// pair's running sum with Kahan's compensated addition; the running sums
// and compensations sit in shared memory, one float2 column per thread.
#include "pair_launch.cuh"

namespace sss {

int dispatch_pairs_kahan(const PairParams& P, cudaStream_t st) { return dispatch_pairs<true>(P, st); }

}  // namespace sss
