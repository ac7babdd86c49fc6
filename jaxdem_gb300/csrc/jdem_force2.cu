// Fused force kernels for 2D systems (templates in jdem_force.cuh).
#include "jdem_force.cuh"

namespace jdem {

template void launch_force_dim<2>(const Bufs& b, int mode, cudaStream_t st);

}  // namespace jdem
