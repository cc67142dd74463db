// Finite-value check of a solver's fields after a run: one grid-stride pass
// per field array, one flag word set by any NaN or Inf (ems_run then
// returns EMS_ERR_NOT_FINITE; the run's traces and fields stay readable).
#include <cuda_runtime.h>

#include "ems_internal.hpp"

namespace ems {

namespace {

template <class T> __global__ void __launch_bounds__(256) nonfinite_kernel(const T *__restrict__ x, size_t n, unsigned *__restrict__ bad)
{
    unsigned b = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b |= isfinite(x[i]) ? 0u : 1u;
    if (__any_sync(0xffffffffu, b) && (threadIdx.x & 31) == 0) atomicOr(bad, 1u);
}

}  // namespace

void Sim::check_finite(std::initializer_list<std::pair<const void *, size_t>> arrays, bool fp64)
{
    if (!d_finite.p) d_finite.alloc(sizeof(unsigned));
    d_finite.zero(stream);
    for (const auto &a : arrays) {
        if (!a.first || a.second == 0) continue;
        const unsigned nb = (unsigned)std::min<size_t>((a.second + 255) / 256, 2048);
        if (fp64) nonfinite_kernel<double><<<nb, 256, 0, stream>>>((const double *)a.first, a.second, d_finite.as<unsigned>());
        else nonfinite_kernel<float><<<nb, 256, 0, stream>>>((const float *)a.first, a.second, d_finite.as<unsigned>());
    }
    EMS_CUDA(cudaGetLastError());
    unsigned bad = 0;
    EMS_CUDA(cudaMemcpyAsync(&bad, d_finite.p, sizeof(bad), cudaMemcpyDeviceToHost, stream));
    EMS_CUDA(cudaStreamSynchronize(stream));
    if (bad) throw Error{EMS_ERR_NOT_FINITE, "NaN or Inf in the fields after the run (unstable time step or non-finite initial fields)"};
}

}  // namespace ems
