// The persistent solver's kernel for double inner solves (device code: persistent_kernel.cuh).
#include "persistent_kernel.cuh"

namespace psgb {

template int persistent_kernel_blocks_per_sm<double>();
template void persistent_kernel_launch<double>(const PersistentArgs<double>&, unsigned, cudaStream_t);

}  // namespace psgb
