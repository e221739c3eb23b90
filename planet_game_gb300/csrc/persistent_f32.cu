// The persistent solver's kernel for float inner solves (device code: persistent_kernel.cuh).
#include "persistent_kernel.cuh"

namespace psgb {

template int persistent_kernel_blocks_per_sm<float>();
template void persistent_kernel_launch<float>(const PersistentArgs<float>&, unsigned, cudaStream_t);

}  // namespace psgb
