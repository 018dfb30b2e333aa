// FP32 particle kernels: positions relative to the cell origin, FP32 push
// with fused multiply-adds, FP64 node accumulation of the deposit.
#include "particles_impl.cuh"

namespace ipg {
template int launch_push<float>(const Geom&, const Pop<float>&, int, cudaStream_t);
template int launch_push_pending<float>(const Geom&, const Pop<float>&, cudaStream_t);
template int launch_inject<float>(const Geom&, const Pop<float>&, double, const double*, const double*, uint64_t,
                                  const uint64_t*, cudaStream_t);
template int launch_place<float>(const Geom&, const Pop<float>&, int32_t*, cudaStream_t);
template int launch_pending_rotate<float>(const Pop<float>&, uint32_t*, cudaStream_t);
}  // namespace ipg
