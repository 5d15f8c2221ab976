// Kernel launches with programmatic dependent launch (PDL).
//
// Every kernel of the engine starts with grid_dep_entry(), which waits until
// the kernel before it in its stream has completed and that kernel's writes
// are visible (griddepcontrol.wait).  ug::launch launches with programmatic
// stream serialisation allowed: the next kernel's launch begins as soon as
// every block of the current one has exited, instead of after the grid's
// completion has been signalled, so its launch and block set-up overlap the
// end of the kernel it follows; under stream capture the launch becomes a
// programmatic graph edge.  Because the wait is the first statement, no
// kernel touches memory before its predecessor is complete: the ordering is
// the plain stream order's.  No kernel triggers its dependents early (waiting
// blocks would then hold SM slots that kernels of the other node streams
// need; measured slower on the 64-chain batch).  Event waits across streams
// and non-kernel nodes keep full dependencies, and a kernel launched without
// the attribute treats the wait as a no-op.
#pragma once
#include <cuda_runtime.h>

#include <utility>

__device__ __forceinline__ void grid_dep_entry() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

namespace ug {

// false when the environment sets UPSIDE_GB300_PDL=0 (plain stream order)
bool pdl_enabled();

template <class... P, class... A>
inline cudaError_t launch(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, A&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl_enabled() ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

}  // namespace ug
