// Standalone pair list of one point set on the device: every (i, j), i < j,
// with |x_i - x_j| < cutoff.  This is the interaction-graph pair search of the
// engine (the reference's PairlistComputation, src/interaction_graph.h:122-157:
// blocks of four set-1 points against all later points) exposed on its own, for callers
// that hold positions in device memory and want the list without building an
// engine.
//
// Layout: positions are n x 3 floats (x, y, z per point), pairs are written
// as int32 (i, j).  The order is the engine's (and the reference's): by
// i / 4, then j, then i % 4.
//
// Two passes with a scan between them: one warp per row of four points counts
// its hits, a single-block scan turns counts into row offsets and the total,
// and the second pass writes each row's pairs at its offset.  The scratch is
// the row counts and row offsets (2 * ceil(n/4) + 1 ints).  A row count is at
// most n; the offsets and the total are summed in 64 bits and saturate at
// INT32_MAX, so a total beyond the int32 range comes back as INT32_MAX (more
// than any capacity) and no write leaves [0, cap).
#include <cuda_runtime.h>

#include <mutex>

#include "graph.h"
#include "launch.cuh"

namespace ug {

template <int PASS>
__global__ void point_pair_kernel(const float* __restrict__ pos, int n, float c2, int* __restrict__ row_count,
                                  const int* __restrict__ row_off, int2* __restrict__ pairs, int cap) {
    grid_dep_entry();
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    int n_warps = (gridDim.x * blockDim.x) >> 5;
    int n_rows = (n + 3) >> 2;
    for (int r = warp; r < n_rows; r += n_warps) {
        int i1s = 4 * r;
        int nl = min(4, n - i1s);
        float ax[4], ay[4], az[4];
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            bool ok = l < nl;
            ax[l] = ok ? pos[3 * (i1s + l)] : 1e20f;
            ay[l] = ok ? pos[3 * (i1s + l) + 1] : 1e20f;
            az[l] = ok ? pos[3 * (i1s + l) + 2] : 1e20f;
        }
        // 64-bit running offset: row offsets saturate at INT_MAX (the scan),
        // so a list too long for int32 writes nothing past the capacity
        long long base = PASS ? row_off[r] : 0;
        int count = 0;
        for (int j0 = i1s + 1; j0 < n; j0 += 32) {
            int j = j0 + lane;
            unsigned mask = 0;
            if (j < n) {
                float bx = pos[3 * j], by = pos[3 * j + 1], bz = pos[3 * j + 2];
#pragma unroll
                for (int l = 0; l < 4; ++l) {
                    if (l >= nl || !(i1s + l < j)) continue;
                    float dx = ax[l] - bx, dy = ay[l] - by, dz = az[l] - bz;
                    float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                    if (d2 < c2) mask |= 1u << l;
                }
            }
            int c = __popc(mask);
            if (PASS == 0) {
                count += c;
            } else {
                int incl = c;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    int y = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += y;
                }
                long long p = base + incl - c;
                for (int l = 0; l < 4; ++l)
                    if (mask & (1u << l)) {
                        if (p >= 0 && p < cap) pairs[p] = make_int2(i1s + l, j);
                        ++p;
                    }
                base += __shfl_sync(0xffffffffu, incl, 31);
            }
        }
        if (PASS == 0) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) count += __shfl_xor_sync(0xffffffffu, count, o);
            if (lane == 0) row_count[r] = count;
        }
    }
}

cudaError_t launch_point_pairs(const float* pos, int n, float cutoff, int* pairs, int cap, int* n_pairs,
                               int* row_count, int* row_off, cudaStream_t st) {
    int n_rows = (n + 3) / 4;
    if (n_rows == 0) return cudaMemsetAsync(n_pairs, 0, sizeof(int), st);
    int blocks = min(8 * 152, (n_rows * 32 + 255) / 256);
    float c2 = cutoff * cutoff;
    int2* p2 = reinterpret_cast<int2*>(pairs);
    ug::launch((point_pair_kernel<0>), blocks, 256, 0, st, pos, n, c2, row_count, row_off, p2, cap);
    launch_scan(row_count, row_off, n_rows, n_pairs, st);
    ug::launch((point_pair_kernel<1>), blocks, 256, 0, st, pos, n, c2, row_count, row_off, p2, cap);
    return cudaGetLastError();
}

// ------------------------------------------------------ no-allocation form --
// Some callers cannot allocate device memory at the moment they need a pair
// list: code running inside a real-time or memory-capped service whose device
// memory is fully reserved up front, callers that must not synchronise the
// device (cudaMalloc/cudaFree can), and host code that owns no allocator of
// its own.  For them the scratch lives in a fixed file-scope device array
// instead of being allocated per call.  Its size bounds the problem: at most
// kNoAllocMaxPoints points (2 * 65536 + 1 ints = 512 KiB of scratch).
//
// Nothing in the scratch needs to start at zero: the counting pass writes
// every row count, and the scan writes every row offset and the total.
// Calls whose kernels can run at the same time on one device (two streams,
// two host threads) share this one array and race; order them on one stream.
constexpr int kNoAllocMaxPoints = 262144;
constexpr int kNoAllocRows = kNoAllocMaxPoints / 4;
static __device__ __align__(256) int g_point_pair_scratch[2 * kNoAllocRows + 1];

int point_pairs_noalloc_max() { return kNoAllocMaxPoints; }

// Device address of the fixed scratch on the current device, looked up once
// per device (the first call on a device does this setup; later calls only
// read the cached pointer).
cudaError_t point_pairs_noalloc_scratch(int** out) {
    constexpr int kMaxDevices = 64;
    static std::mutex mu;
    static int* addr[kMaxDevices] = {};
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_point_pair_scratch);
        if (e != cudaSuccess) return e;
        addr[dev] = static_cast<int*>(p);
    }
    *out = addr[dev];
    return cudaSuccess;
}

}  // namespace ug
