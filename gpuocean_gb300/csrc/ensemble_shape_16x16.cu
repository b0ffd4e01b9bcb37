// The batched ensemble kernel with 16x16 output tiles.
#include "ensemble.cuh"

namespace goc {
template int ensemble_configure_shape<16, 16>(const Ensemble*, int*);
template int ensemble_launch_shape<16, 16>(Ensemble*, int, cudaStream_t, const FusedNoise*);
}  // namespace goc
