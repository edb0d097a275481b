// Programmatic dependent launch for the kernels of a replayed time step.
//
// A kernel launched by pdl_launch may be scheduled while the previous kernel of
// the stream is still finishing; it must call pdl_wait() before its first memory
// access, which returns once the previous kernel has completed and its writes are
// visible (griddepcontrol.wait; a no-op for an ordinary launch).  The previous
// kernel's CTAs trigger the launch implicitly as they exit: an explicit trigger on
// entry let the next kernels' CTAs hold the SMs while they waited, and was slower.
// ODIS_PDL=0 launches in plain stream order.
#pragma once

#include <cuda_runtime.h>

#include <cstdlib>

namespace odis {

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

inline bool pdl_on()
{
    static const bool on = [] {
        const char* e = std::getenv("ODIS_PDL");
        return !(e && e[0] == '0');
    }();
    return on;
}

// Returns the launch status.  If the driver refuses the attributed launch (for
// instance under a capture mode that does not take it), the kernel is launched
// again in plain stream order and that launch's status is returned.
template <typename... KArgs, typename... Args>
inline cudaError_t pdl_launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl_on() ? 1 : 0;
    cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
    if (e != cudaSuccess && cfg.numAttrs) {
        (void)cudaGetLastError();          // the refused launch's error, replaced by the retry's
        cfg.numAttrs = 0;
        e = cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
    }
    return e;
}

}  // namespace odis
