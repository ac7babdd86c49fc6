// Fused force kernels for 3D systems (templates in jdem_force.cuh).
#include "jdem_force.cuh"

namespace jdem {

template void launch_force_dim<3>(const Bufs& b, int mode, cudaStream_t st);

}  // namespace jdem
