// The batched ensemble kernel with 32x24 output tiles.
#include "ensemble.cuh"

namespace goc {
template int ensemble_configure_shape<32, 24>(const Ensemble*, int*);
template int ensemble_launch_shape<32, 24>(Ensemble*, int, cudaStream_t, const FusedNoise*);
}  // namespace goc
