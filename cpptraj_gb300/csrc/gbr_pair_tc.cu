// gbr_pair_tc.cu -- tensor-core (tcgen05) pair contraction.  Placeholder until
// the sm_103a kernel lands: reports the precision as unsupported.
#include "gbr_internal.h"

namespace gbr {
int tc_supported(int) { return 0; }
cudaError_t run_pairs_tc(const TcLaunch&, cudaStream_t) { return cudaErrorNotSupported; }
}  // namespace gbr
