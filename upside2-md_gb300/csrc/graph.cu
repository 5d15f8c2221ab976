// Interaction-graph kernels (pair search in the reference's edge order, edge
// evaluation, sensitivity scatter), the batch prefix scan, and the rotamer
// belief-propagation kernels.  sm_103a, FP32 arithmetic, FP64 energy sums.
//
// Reference behaviour restated here:
//   pair search / edge order   src/interaction_graph.h:51-258
//   edge values / adjoint      src/interaction_graph.h:445-564
//   quadspline                 src/bead_interaction.h:31-85
//   protein hbond edge         src/hbond.cpp:158-246
//   hbond coverage edge        src/hbond.cpp:249-294
//   environment coverage edges src/environment.cpp:114-228
//   rotamer BP                 src/rotamer.cpp:239-302, :425-569, :854-1162
#include <cooperative_groups.h>
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstdlib>

#include "dev_math.cuh"
#include "launch.cuh"
#include "graph.h"
#include "warm.h"

namespace ug {

namespace cg = cooperative_groups;

// ---------------------------------------------------------------- scan ---
// Exclusive scan of n ints into out[0..n] (out[n] = total) by one 1024-thread
// block, in tiles of SCAN_K x 1024: a tile is loaded into shared memory with
// coalesced, independent loads, each thread scans its SCAN_K consecutive
// elements there, a block-level scan of the thread sums (plus the carry of
// the tiles before) gives their offsets, and the tile is stored back
// coalesced.  Shared-memory indices are padded by one word per 32, so the
// threads' runs of SCAN_K fall into different banks.
constexpr int SCAN_K = 8, SCAN_TILE = 1024 * SCAN_K;
__device__ __forceinline__ int scan_pad(int i) { return i + (i >> 5); }

__global__ void __launch_bounds__(1024) scan_kernel(const int* __restrict__ in, int* __restrict__ out, int n,
                                                    int* total_out, const int* __restrict__ skip_unless, int cap,
                                                    int* status, int bit) {
    grid_dep_entry();
    if (skip_unless && !*skip_unless) return;
    // sums are carried in 64 bits and stored saturated at INT_MAX, so a total
    // beyond the int range reads as "larger than any capacity" rather than
    // wrapping to a negative offset
    __shared__ long long warp_sums[32];
    __shared__ int sm[SCAN_TILE + SCAN_TILE / 32];
    auto sat = [](long long x) { return int(x < 2147483647LL ? x : 2147483647LL); };
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    long long carry = 0;
    for (int base = 0; base < n; base += SCAN_TILE) {  // block-uniform
        const int m = min(SCAN_TILE, n - base);
#pragma unroll
        for (int k = 0; k < SCAN_K; ++k) {
            const int i = k * 1024 + t;
            sm[scan_pad(i)] = i < m ? in[base + i] : 0;
        }
        __syncthreads();
        int x[SCAN_K];
        long long s = 0;
#pragma unroll
        for (int j = 0; j < SCAN_K; ++j) {
            x[j] = sm[scan_pad(t * SCAN_K + j)];
            s += x[j];
        }
        // block exclusive scan of s
        long long v = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            long long y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        if (lane == 31) warp_sums[w] = v;
        __syncthreads();
        if (w == 0) {
            long long ws = warp_sums[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                long long y = __shfl_up_sync(0xffffffffu, ws, o);
                if (lane >= o) ws += y;
            }
            warp_sums[lane] = ws;
        }
        __syncthreads();
        long long excl = carry + v - s + (w ? warp_sums[w - 1] : 0);
        const long long tile_total = warp_sums[31];
        // each thread rewrites only the run it read
#pragma unroll
        for (int j = 0; j < SCAN_K; ++j) {
            sm[scan_pad(t * SCAN_K + j)] = sat(excl);
            excl += x[j];
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < SCAN_K; ++k) {
            const int i = k * 1024 + t;
            if (i < m) out[base + i] = sm[scan_pad(i)];
        }
        carry += tile_total;
        __syncthreads();  // sm and warp_sums are reused by the next tile
    }
    if (t == 0) {
        out[n] = sat(carry);
        if (total_out) {
            // with a capacity: a total beyond it is flagged and capped (the
            // fill pass writes no further)
            int tot = sat(carry);
            if (cap >= 0 && tot > cap) {
                atomicOr(status, bit);
                tot = cap;
            }
            *total_out = tot;
        }
    }
}

void launch_scan(const int* in, int* out, int n, int* total_out, cudaStream_t st, const int* skip_unless, int cap,
                 int* status, int bit) {
    ug::launch(scan_kernel, 1, 1024, 0, st, in, out, n, total_out, skip_unless, cap, status, bit);
}

// blocks of the grid-stride kernels over edges and entries: their loops are
// chains of dependent loads, so more warps in flight shorten them
constexpr int EDGE_BLOCKS = 8 * 152;

// --------------------------------------------------------- pair search ---
__global__ void pack_kernel(const int* __restrict__ loc, const float* __restrict__ in, int w, int n,
                            float4* __restrict__ x) {
    grid_dep_entry();
    for (int i = grid_stride_start(); i < n; i += grid_stride()) {
        const float* p = in + size_t(loc[i]) * w;
        x[i] = make_float4(p[0], p[1], p[2], 0.f);
    }
}

void launch_pack_positions(const DGraph& g, cudaStream_t st) {
    if (g.n1) ug::launch(pack_kernel, min(1024, (g.n1 + 255) / 256), 256, 0, st, g.loc1, g.in1, g.w1, g.n1, g.x1);
    if (!g.symmetric && g.n2) ug::launch(pack_kernel, min(1024, (g.n2 + 255) / 256), 256, 0, st, g.loc2, g.in2, g.w2, g.n2, g.x2);
}

// One warp per row (4 consecutive set-1 elements of one system).  Pass 0
// counts hits; pass 1 writes them in (i2, lane) order at the row's scanned
// offset, which reproduces the reference's edge order exactly.
//
// CACHED: the search fills the candidate cache instead of the edge list: it
// runs only for the rows of systems flagged for a rebuild, with cutoff +
// buffer, and writes each system's candidates into its own cache segment
// (the reference's cache rebuild, src/interaction_graph.h:96-157).
// minimum image of a displacement in the periodic box (no change when open)
__device__ __forceinline__ float min_image1(float d, float L) { return L > 0.f ? d - L * rintf(d / L) : d; }
__device__ __forceinline__ f3 min_image(f3 d, const float* box) {
    return mk(min_image1(d.x, box[0]), min_image1(d.y, box[1]), min_image1(d.z, box[2]));
}
__device__ __forceinline__ float pair_d2(float4 a, float4 b, const float* box) {
    float dx = min_image1(a.x - b.x, box[0]), dy = min_image1(a.y - b.y, box[1]), dz = min_image1(a.z - b.z, box[2]);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// Partner tiles in shared memory: a block takes 8 consecutive rows (one per
// warp), and for the union of their candidate ranges loads tiles of 256
// partners (position and id) into shared memory once; each warp then scans
// the part of every tile that lies in its own row's range, in increasing j,
// so the rows' hits come out in exactly the order of a warp scanning its
// range alone.
constexpr int PAIR_TILE = 256;
__device__ void cache_commit(DGraph& g);
template <int PASS, bool CACHED>
__global__ void __launch_bounds__(256) pair_kernel(DGraph g) {
    grid_dep_entry();
    if (CACHED && !*g.any_flag) return;  // no system rebuilt in this evaluation
    if (PASS == 1 && CACHED && blockIdx.x == 0) cache_commit(g);  // counts and tiles for the refine
    __shared__ float4 s_x[PAIR_TILE];
    __shared__ int s_id[PAIR_TILE];
    __shared__ int s_lo, s_hi;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const float rc = CACHED ? g.cutoff + g.buffer : g.cutoff;
    const float c2 = rc * rc;
    const float4* X2 = g.symmetric ? g.x1 : g.x2;
    const int* ID2 = g.symmetric ? g.id1 : g.id2;
    const int n_rb = (g.n_rows + 7) >> 3;
    for (int rb = blockIdx.x; rb < n_rb; rb += gridDim.x) {  // block-uniform
        const int r = rb * 8 + warp;
        bool active = r < g.n_rows;
        int i1s = 0, i1e = 0, sys = 0, i2s = 0, i2e = 0;
        if (active) {
            i1s = g.row_i1[r];
            i1e = g.row_i1_end[r];
            if (CACHED) {
                sys = g.sys1[i1s];
                active = g.sys_flag[sys] != 0;  // warp-uniform
            }
            i2s = g.row_i2[r];
            i2e = g.row_i2_end[r];
        }
        if (threadIdx.x == 0) {
            s_lo = 0x7fffffff;
            s_hi = -1;
        }
        __syncthreads();
        if (active && lane == 0 && i2s < i2e) {
            atomicMin(&s_lo, i2s);
            atomicMax(&s_hi, i2e);
        }
        __syncthreads();
        const int lo = s_lo, hi = s_hi;
        float4 a[4];
        int ida[4];
        const int nl = active ? min(4, i1e - i1s) : 0;
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            a[l] = l < nl ? g.x1[i1s + l] : make_float4(1e20f, 1e20f, 1e20f, 0.f);
            ida[l] = l < nl ? g.id1[i1s + l] : 0;
        }
        int base = 0, lim = g.cap;
        int2* out = g.edges;
        if (PASS && active) {
            if (CACHED) {
                int seg = g.cache_off[sys];
                base = seg + g.row_off[r] - g.row_off[g.sys_first_row[sys]];
                lim = g.cache_off[sys + 1];
                out = g.cache_edges;
            } else {
                base = g.row_off[r];
            }
        }
        int count = 0;
        for (int t0 = lo; t0 < hi; t0 += PAIR_TILE) {  // block-uniform (lo > hi when no row is active)
            __syncthreads();  // the previous tile is consumed
            const int jt = t0 + threadIdx.x;
            if (jt < hi) {
                s_x[threadIdx.x] = X2[jt];
                s_id[threadIdx.x] = ID2[jt];
            }
            __syncthreads();
            if (!active) continue;
            const int c0 = max(t0, i2s), c1 = min(t0 + PAIR_TILE, i2e);
            for (int j0 = c0; j0 < c1; j0 += 32) {  // warp-uniform
                const int j = j0 + lane;
                unsigned mask = 0;
                if (j < c1) {
                    const float4 bx = s_x[j - t0];
                    const int idb = s_id[j - t0];
#pragma unroll
                    for (int l = 0; l < 4; ++l) {
                        if (l >= nl) break;
                        if (g.symmetric && !(i1s + l < j)) continue;
                        if (pair_d2(a[l], bx, g.box) < c2 && acceptable_ids(g.excl, ida[l], idb)) mask |= 1u << l;
                    }
                }
                const int c = __popc(mask);
                if (PASS == 0) {
                    count += c;
                } else {
                    int incl = c;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        int y = __shfl_up_sync(0xffffffffu, incl, o);
                        if (lane >= o) incl += y;
                    }
                    int pos = base + incl - c;
                    for (int l = 0; l < 4; ++l)
                        if (mask & (1u << l)) {
                            if (pos < lim) out[pos] = make_int2(i1s + l, j);
                            ++pos;
                        }
                    base += __shfl_sync(0xffffffffu, incl, 31);
                }
            }
        }
        if (PASS == 0 && active) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) count += __shfl_xor_sync(0xffffffffu, count, o);
            if (lane == 0) g.row_count[r] = count;
        }
        __syncthreads();  // s_lo / s_hi are reset for the next row block
    }
    if (PASS == 1 && CACHED) {
        // the rebuilt systems' positions become their new reference positions
        // (the search reads x1 / x2 only)
        const int n = g.n1 + (g.symmetric ? 0 : g.n2);
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
            const bool first = i < g.n1;
            const int k = first ? i : i - g.n1;
            if (!g.sys_flag[first ? g.sys1[k] : g.sys2[k]]) continue;
            if (first) g.xc1[k] = g.x1[k];
            else g.xc2[k] = g.x2[k];
        }
    }
}


// ----------------------------------------------------- candidate cache ---
// A system's cache is rebuilt when any of its elements moved more than half
// the buffer since its last rebuild, when its segment overflowed at the last
// rebuild, or when a rebuild of every system was requested
// (src/interaction_graph.h:51-91: same bound, same comparison).
// This kernel also packs the positions the search reads.  The flags it sets
// were cleared, down to the systems whose segment overflowed, by the
// previous evaluation's refine (cache_refine_kernel<1>, block 0).
__global__ void cache_check_kernel(DGraph g) {
    grid_dep_entry();
    for (int i = grid_stride_start(); i < g.cov_n; i += grid_stride())  // coverage sums
        g.cov_out[size_t(i) * g.cov_w + g.cov_w - 1] = 0.f;
    if (*g.cache_force) {
        for (int s = grid_stride_start(); s < g.n_sys; s += grid_stride()) g.sys_flag[s] = 1;
        if (blockIdx.x == 0 && threadIdx.x == 0) *g.any_flag = 1;
    }
    float h = 0.5f * ((g.cutoff + g.buffer) - g.cutoff);
    float lim = h * h;
    int n = g.n1 + (g.symmetric ? 0 : g.n2);
    for (int i = grid_stride_start(); i < n; i += grid_stride()) {
        bool first = i < g.n1;
        int k = first ? i : i - g.n1;
        int sys = first ? g.sys1[k] : g.sys2[k];
        const float* p = first ? g.in1 + size_t(g.loc1[k]) * g.w1 : g.in2 + size_t(g.loc2[k]) * g.w2;
        const float4 x = make_float4(p[0], p[1], p[2], 0.f);
        if (first) g.x1[k] = x;
        else g.x2[k] = x;
        float4 c = first ? g.xc1[k] : g.xc2[k];
        float dx = x.x - c.x, dy = x.y - c.y, dz = x.z - c.z;
        if (lim < dx * dx + dy * dy + dz * dz) {
            g.sys_flag[sys] = 1;
            *g.any_flag = 1;
        }
    }
}

// after the rebuild search: per system candidate counts (capped by the
// segment, overflow flagged), then the refine pass's tile prefix over systems
// and the end of a rebuild-everything request; run by one block (block 0 of
// the rebuild's fill pass, from the scanned row offsets)
__device__ void cache_commit(DGraph& g) {
    for (int s = threadIdx.x; s < g.n_sys; s += blockDim.x) {
        if (!g.sys_flag[s]) continue;
        atomicAdd(g.rebuilds, 1ull);
        int cnt = g.row_off[g.sys_first_row[s + 1]] - g.row_off[g.sys_first_row[s]];
        int cap = g.cache_off[s + 1] - g.cache_off[s];
        g.sys_over[s] = cnt > cap;
        if (cnt > cap) {
            atomicOr(g.status, ST_EDGE_OVERFLOW);
            cnt = cap;
        }
        g.cache_n[s] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        *g.cache_force = 0;
        int t = 0;
        for (int s = 0; s < g.n_sys; ++s) {
            g.active_off[s] = t;
            t += (g.cache_n[s] + CACHE_TILE - 1) / CACHE_TILE;
        }
        g.active_off[g.n_sys] = t;
    }
}

// Refine: the edges are the cached candidates now within the cutoff, in
// cache order (src/interaction_graph.h:203-258).  One block per active tile
// of CACHE_TILE candidates (4 per thread); pass 0 counts each tile's hits,
// a scan over tiles gives offsets, pass 1 writes them in order.
template <int PASS>
__global__ void __launch_bounds__(256) cache_refine_kernel(DGraph g) {
    grid_dep_entry();
    __shared__ int warp_sum[8];
    if (PASS == 1 && blockIdx.x == 0) {
        // the next evaluation's rebuild flags: the systems whose segment
        // overflowed (nothing later in this evaluation reads the flags)
        __shared__ int s_any;
        if (threadIdx.x == 0) s_any = 0;
        __syncthreads();
        for (int s = threadIdx.x; s < g.n_sys; s += blockDim.x) {
            const int o = g.sys_over[s];
            g.sys_flag[s] = o;
            if (o) s_any = 1;
        }
        __syncthreads();
        if (threadIdx.x == 0) *g.any_flag = s_any;
    }
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int n_active = g.active_off[g.n_sys];
    const float c2 = g.cutoff * g.cutoff;
    const float4* X2 = g.symmetric ? g.x1 : g.x2;
    for (int t = blockIdx.x; t < g.max_tiles; t += gridDim.x) {
        if (t >= n_active) {  // block-uniform
            if (PASS == 0 && tid == 0) g.tile_count[t] = 0;
            continue;
        }
        int a = 0, z = g.n_sys;  // system s with active_off[s] <= t < active_off[s+1]
        while (z - a > 1) {
            int m = (a + z) >> 1;
            if (g.active_off[m] <= t) a = m; else z = m;
        }
        const int s = a;
        const int first = (t - g.active_off[s]) * CACHE_TILE + 4 * tid;  // within the segment
        const int n = g.cache_n[s];
        const int2* ce = g.cache_edges + g.cache_off[s];
        unsigned mask = 0;
        int2 ij[4];
        unsigned char* tm = g.refine_mask + size_t(t) * (CACHE_TILE / 4) + tid;
        if (PASS == 0) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                int k = first + q;
                if (k < n) {
                    const int2 c = ce[k];
                    if (pair_d2(g.x1[c.x], X2[c.y], g.box) < c2) mask |= 1u << q;
                }
            }
            *tm = (unsigned char)mask;  // the fill pass writes these candidates
        } else {
            mask = *tm;
#pragma unroll
            for (int q = 0; q < 4; ++q) ij[q] = (mask >> q & 1u) ? ce[first + q] : make_int2(0, 0);
        }
        int c = __popc(mask);
        int incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) warp_sum[warp] = incl;
        __syncthreads();
        if (PASS == 0) {
            if (tid == 0) {
                int tot = 0;
                for (int w = 0; w < 8; ++w) tot += warp_sum[w];
                g.tile_count[t] = tot;
            }
        } else {
            int pos = g.tile_off[t] + incl - c;
            for (int w = 0; w < warp; ++w) pos += warp_sum[w];
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (mask & (1u << q)) {
                    if (pos < g.cap) g.edges[pos] = ij[q];
                    ++pos;
                }
        }
        __syncthreads();  // warp_sum is reused by the next tile
    }
}

// Launches per evaluation: full search 4 (pack, count, scan with the edge
// capacity check, fill); cached 7 (movement check with the position packing,
// rebuild count, scan, rebuild fill with the commit and the new reference
// positions, refine count, scan with the capacity check, refine fill with
// the next evaluation's rebuild flags).
__global__ void cov_zero_kernel(DGraph g) {
    grid_dep_entry();
    for (int i = grid_stride_start(); i < g.cov_n; i += grid_stride()) g.cov_out[size_t(i) * g.cov_w + g.cov_w - 1] = 0.f;
}

void launch_pairs(const DGraph& g, cudaStream_t st) {
    // coverage sums: zeroed by the movement check on the cached path
    if (g.cov_out && (g.n_rows == 0 || !g.cached)) ug::launch(cov_zero_kernel, EDGE_BLOCKS, 256, 0, st, g);
    if (g.n_rows == 0) {
        launch_pack_positions(g, st);
        cudaMemsetAsync(g.n_edge, 0, sizeof(int), st);
        cudaMemsetAsync(g.row_off, 0, sizeof(int), st);
        return;
    }
    int blocks = min(EDGE_BLOCKS, (g.n_rows + 7) / 8);
    if (!g.cached) {
        launch_pack_positions(g, st);
        ug::launch((pair_kernel<0, false>), blocks, 256, 0, st, g);
        launch_scan(g.row_count, g.row_off, g.n_rows, g.n_edge, st, nullptr, g.cap, g.status);
        ug::launch((pair_kernel<1, false>), blocks, 256, 0, st, g);
        return;
    }
    int ne = g.n1 + (g.symmetric ? 0 : g.n2);
    int eb = min(1024, (ne + 255) / 256);
    ug::launch(cache_check_kernel, eb, 256, 0, st, g);
    ug::launch((pair_kernel<0, true>), blocks, 256, 0, st, g);
    launch_scan(g.row_count, g.row_off, g.n_rows, nullptr, st, g.any_flag);
    ug::launch((pair_kernel<1, true>), blocks, 256, 0, st, g);
    int rblocks = min(8 * 152, g.max_tiles);
    ug::launch((cache_refine_kernel<0>), rblocks, 256, 0, st, g);
    launch_scan(g.tile_count, g.tile_off, g.max_tiles, g.n_edge, st, nullptr, g.cap, g.status);
    ug::launch((cache_refine_kernel<1>), rblocks, 256, 0, st, g);
}

// ------------------------------------------------------ edge evaluation ---
__device__ float quadspline(int n_ka, int n_k, float inv_dtheta, float inv_dx, const float* p, const float* x1,
                            const float* x2, float* d1, float* d2, const float* box) {
    f3 disp = min_image(ld3(x2) - ld3(x1), box), r1 = ld3(x1 + 3), r2 = ld3(x2 + 3);
    float dist2 = mag2(disp), inv_dist = rsqrtf(dist2);
    float dc = dist2 * (inv_dist * inv_dx);
    f3 u = disp * inv_dist;
    float c1 = dot(r1, u), c2 = -dot(r2, u);
    float a1v, a1d, a2v, a2d, wv, wd, nv, nd;
    deboor(p, (c1 + 1.f) * inv_dtheta + 1.f, a1v, a1d);
    deboor(p + n_ka, (c2 + 1.f) * inv_dtheta + 1.f, a2v, a2d);
    clamped(p + 2 * n_ka, dc, n_k, wv, wd);
    clamped(p + 2 * n_ka + n_k, dc, n_k, nv, nd);
    float aw = a1v * a2v;
    float rad = inv_dx * (wd + aw * nd);
    float ad1 = inv_dtheta * a1d * a2v * nv;
    float ad2 = inv_dtheta * a1v * a2d * nv;
    f3 rXX = r1 * ad1 - r2 * ad2;
    f3 ddir = (rXX - u * dot(u, rXX)) * inv_dist;
    f3 dd = u * rad + ddir;
    st3(d1, -dd);
    st3(d1 + 3, u * ad1);
    st3(d2, dd);
    st3(d2 + 3, u * (-ad2));
    return wv + aw * nv;
}

__device__ __forceinline__ bool phb_in_angle(const float* H, const float* O, const float* box) {
    f3 HO = min_image(ld3(H) - ld3(O), box);
    float m2 = mag2(HO) + 1e-6f;
    f3 rHO = HO * rsqrtf(m2);
    return (dot(rHO, ld3(O + 3)) > 0.f) && (-dot(rHO, ld3(H + 3)) > 0.f);
}

template <int KIND>
__device__ float edge_value(const DGraph& g, const float* p, const float* a, const float* b, float* da, float* db,
                            bool active) {
    if (KIND == IK_ROTAMER) return quadspline(15, 12, 6.f, 1.f / 0.7f, p, a, b, da, db, g.box);
    if (KIND == IK_HBCOV) {
        float cov = quadspline(15, 10, 6.f, 1.f / 0.625f, p, a, b, da, db, g.box);
        float om = 1.f - a[6];
        float pre = om * om;
#pragma unroll
        for (int i = 0; i < 6; ++i) { da[i] *= pre; db[i] *= pre; }
        da[6] = -cov * om * 2.f;
        return pre * cov;
    }
    if (KIND == IK_PHB) {
        f3 rHN = ld3(a + 3), rOC = ld3(b + 3);
        f3 HO = min_image(ld3(a) - ld3(b), g.box);
        float m2 = mag2(HO) + 1e-6f, inv = rsqrtf(m2), mg = m2 * inv;
        f3 rHO = HO * inv;
        float dHOC = dot(rHO, rOC), dOHN = -dot(rHO, rHN);
        float hb = 0.f;
        f3 dH = mk(0, 0, 0), drHN = mk(0, 0, 0), drOC = mk(0, 0, 0);
        if (active) {
            float ov, od, iv, id_, a1v, a1d, a2v, a2d;
            logistic((p[2] - mg) * p[3], ov, od);
            logistic((mg - p[0]) * p[1], iv, id_);
            float rv = ov * iv, rd = -p[3] * od * iv + p[1] * id_ * ov;
            logistic((dHOC - p[4]) * p[5], a1v, a1d);
            a1d *= p[5];
            logistic((dOHN - p[4]) * p[5], a2v, a2d);
            a2d *= p[5];
            hb = rv * a1v * a2v;
            float c0 = rd * a1v * a2v, c1 = rv * a1d * a2v, c2 = -rv * a1v * a2d;
            drOC = rHO * c1;
            drHN = rHO * c2;
            dH = rHO * c0 + (rOC - rHO * dHOC) * (c1 * inv) + (rHN + rHO * dOHN) * (c2 * inv);
        }
        float hb_log = (1.f <= hb) ? 100.f : -logf(1.f - hb);
        float pre = fminf(1.f / (1.f - hb), 1e5f);
        st3(da, dH * pre);
        st3(da + 3, drHN * pre);
        st3(db, dH * (-pre));
        st3(db + 3, drOC * pre);
        return hb_log;
    }
    if (KIND == IK_ENVCOV || KIND == IK_HBENV) {
        f3 disp = min_image(ld3(b) - ld3(a), g.box), r1 = ld3(a + 3);
        float prob = KIND == IK_ENVCOV ? b[3] : 1.f;
        float d2 = mag2(disp), inv = rsqrtf(d2), dist = d2 * inv;
        f3 u = disp * inv;
        float dp = dot(u, r1), rv, rd, av, ad;
        csig(dist - p[0], p[1], rv, rd);
        csig(p[2] - dp, p[3], av, ad);
        f3 dd = (u * (rd * av) - (r1 - u * dp) * (rv * ad * inv)) * prob;
        st3(da + 3, u * (-prob * rv * ad));
        st3(da, -dd);
        st3(db, dd);
        float score = rv * av;
        if (KIND == IK_ENVCOV) {
            db[3] = score;
            return prob * score;
        }
        db[3] = db[4] = db[5] = 0.f;
        return score;
    }
    return 0.f;
}

// the coverage row an edge adds into
__device__ __forceinline__ int cov_row(const DGraph& g, int2 ij) {
    return g.cov_by_first ? (g.cov_aa2 ? ij.x * g.cov_n_aa + g.cov_aa2[ij.y] : ij.x) : ij.y;
}

template <int KIND>
__global__ void edge_eval_kernel(DGraph g, const int* __restrict__ edge_sys_start, const int* __restrict__ edge_sys_end) {
    grid_dep_entry();
    int ne = *g.n_edge;
    int dw = g.d1 + g.d2;
    for (int e = grid_stride_start(); e < ne; e += grid_stride()) {
        int2 ij = g.edges[e];
        const float* a = g.in1 + size_t(g.loc1[ij.x]) * g.w1;
        const float* b = g.in2 + size_t(g.loc2[ij.y]) * g.w2;
        const float* p = g.param + (size_t(g.type1[ij.x]) * g.n_type2 + g.type2[ij.y]) * g.n_param;
        bool active = true;
        if (KIND == IK_PHB) {
            // lanes of a group of 4 consecutive edges of one system are
            // evaluated together; a group with no edge inside the angular
            // cutoff gives zero for all its edges (src/hbond.cpp:207-213)
            int s = g.sys1[ij.x];
            int st = edge_sys_start[s], en = edge_sys_end[s];
            int g0 = st + ((e - st) & ~3);
            active = false;
            for (int k = g0; k < min(g0 + 4, en); ++k) {
                int2 q = g.edges[k];
                active |= phb_in_angle(g.in1 + size_t(g.loc1[q.x]) * g.w1, g.in2 + size_t(g.loc2[q.y]) * g.w2, g.box);
            }
        }
        float* da = g.deriv + size_t(e) * dw;
        const float v = edge_value<KIND>(g, p, a, b, da, da + g.d1, active);
        g.value[e] = v;
        if (KIND == IK_HBCOV || KIND == IK_ENVCOV || KIND == IK_HBENV) {
            if (g.cov_out) atomicAdd(g.cov_out + cov_row(g, ij), v);
        } else if (KIND == IK_PHB) {
            if (g.phb_row1) {
                atomicAdd(g.cov_out + 7 * size_t(g.phb_row1[ij.x]) + 6, v);
                atomicAdd(g.cov_out + 7 * size_t(g.phb_row2[ij.y]) + 6, v);
            }
        }
    }
}

__global__ void edge_sys_range_kernel(DGraph g, int* start, int* end) {
    grid_dep_entry();
    for (int s = grid_stride_start(); s < g.n_sys; s += grid_stride()) {
        start[s] = min(g.row_off[g.sys_first_row[s]], g.cap);
        end[s] = min(g.row_off[g.sys_first_row[s + 1]], g.cap);
    }
}

// per-system edge ranges from the edge list itself (edges are in system order)
__global__ void edge_sys_bounds_kernel(DGraph g, int* start, int* end) {
    grid_dep_entry();
    int n = min(*g.n_edge, g.cap);
    for (int e = grid_stride_start(); e < n; e += grid_stride()) {
        int s = g.sys1[g.edges[e].x];
        if (e == 0 || g.sys1[g.edges[e - 1].x] != s) start[s] = e;
        if (e == n - 1 || g.sys1[g.edges[e + 1].x] != s) end[s] = e + 1;
    }
}

void launch_edge_eval(const DGraph& g, int* sys_start, int* sys_end, cudaStream_t st) {
    int blocks = EDGE_BLOCKS;
    if (g.kind == IK_PHB) {
        if (g.cached) {
            cudaMemsetAsync(sys_start, 0, sizeof(int) * size_t(g.n_sys), st);
            cudaMemsetAsync(sys_end, 0, sizeof(int) * size_t(g.n_sys), st);
            ug::launch(edge_sys_bounds_kernel, blocks, 256, 0, st, g, sys_start, sys_end);
        } else {
            ug::launch(edge_sys_range_kernel, 1, 256, 0, st, g, sys_start, sys_end);
        }
    }
    switch (g.kind) {
        case IK_ROTAMER: ug::launch((edge_eval_kernel<IK_ROTAMER>), blocks, 256, 0, st, g, sys_start, sys_end); break;
        case IK_HBCOV: ug::launch((edge_eval_kernel<IK_HBCOV>), blocks, 256, 0, st, g, sys_start, sys_end); break;
        case IK_PHB: ug::launch((edge_eval_kernel<IK_PHB>), blocks, 256, 0, st, g, sys_start, sys_end); break;
        case IK_ENVCOV: ug::launch((edge_eval_kernel<IK_ENVCOV>), blocks, 256, 0, st, g, sys_start, sys_end); break;
        case IK_HBENV: ug::launch((edge_eval_kernel<IK_HBENV>), blocks, 256, 0, st, g, sys_start, sys_end); break;
        default: break;
    }
}

// Adds each lane's n values into row `key` of dst (row stride w; key < 0:
// nothing).  Lanes holding the same key in a run of consecutive lanes (edges
// of one set-1 element, which the pair search emits together) are summed
// first with suffix sums over the run, and the run's first lane adds once.
// Every lane of the warp calls it.
constexpr int SCATTER_MAXD = 8;
__device__ __forceinline__ void warp_run_add(float* dst, int w, int key, const float* v_in, int n) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int prev = __shfl_up_sync(full, key, 1);
    const unsigned heads = __ballot_sync(full, lane == 0 || prev != key);
    const unsigned later = heads & ~((2u << lane) - 1u);  // run heads after this lane
    const int run_end = later ? __ffs(later) - 1 : 32;    // first lane past this lane's run
    float v[SCATTER_MAXD];
#pragma unroll
    for (int d = 0; d < SCATTER_MAXD; ++d) v[d] = d < n ? v_in[d] : 0.f;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const bool same = lane + off < run_end;
#pragma unroll
        for (int d = 0; d < SCATTER_MAXD; ++d) {
            float t = __shfl_down_sync(full, v[d], off);
            if (same && d < n) v[d] += t;
        }
    }
    if ((heads >> lane & 1u) && key >= 0) {
        float* p = dst + size_t(key) * w;
        for (int d = 0; d < n; ++d) atomicAdd(p + d, v[d]);
    }
}

__global__ void edge_scatter_kernel(DGraph g) {
    grid_dep_entry();
    const int ne = *g.n_edge;
    const int dw = g.d1 + g.d2;
    const bool runs = g.d1 <= SCATTER_MAXD;
    // warp-uniform trip count: every lane takes part in the run sums
    const int stride = grid_stride(), first = grid_stride_start() - (threadIdx.x & 31);
    for (int e0 = first; e0 < ne; e0 += stride) {
        const int e = e0 + (threadIdx.x & 31);
        float s = 0.f;
        if (e < ne) {
            if (g.phb_row1) {  // protein hbonds: from the donor's and the acceptor's scores
                const int2 ij = g.edges[e];
                const size_t a = 7 * size_t(g.phb_row1[ij.x]) + 6, c = 7 * size_t(g.phb_row2[ij.y]) + 6;
                s = g.cov_sens[a] * (1.f - g.cov_out[a]) + g.cov_sens[c] * (1.f - g.cov_out[c]);
                g.esens[e] = s;
            } else if (g.cov_sens) {  // a coverage graph: the edge's sensitivity is its row's
                s = g.cov_sens[cov_row(g, g.edges[e])];
                g.esens[e] = s;
            } else {
                s = g.esens[e];
            }
        }
        int key = -1;
        float v1[SCATTER_MAXD];
        if (s != 0.f) {
            int2 ij = g.edges[e];
            const float* da = g.deriv + size_t(e) * dw;
            key = g.loc1[ij.x];
            float* s2 = g.sens2 + size_t(g.loc2[ij.y]) * g.w2;
            for (int d = 0; d < g.d2; ++d) atomicAdd(s2 + d, s * da[g.d1 + d]);
            if (runs) {
#pragma unroll
                for (int d = 0; d < SCATTER_MAXD; ++d) v1[d] = d < g.d1 ? s * da[d] : 0.f;
            } else {
                float* s1 = g.sens1 + size_t(key) * g.w1;
                for (int d = 0; d < g.d1; ++d) atomicAdd(s1 + d, s * da[d]);
            }
        } else {
#pragma unroll
            for (int d = 0; d < SCATTER_MAXD; ++d) v1[d] = 0.f;
        }
        if (runs) warp_run_add(g.sens1, g.w1, key, v1, g.d1);
    }
}

void launch_edge_scatter(const DGraph& g, cudaStream_t st) {
    ug::launch(edge_scatter_kernel, EDGE_BLOCKS, 256, 0, st, g);
}

// dE/dparam for the quadspline graphs, accumulated per type pair with the
// current edge sensitivities (src/interaction_graph.h:406-416, :498-550,
// src/bead_interaction.h:87-131)
__global__ void param_deriv_kernel(DGraph g, float* __restrict__ out) {
    grid_dep_entry();
    int ne = *g.n_edge;
    for (int e = grid_stride_start(); e < ne; e += grid_stride()) {
        float s = g.esens[e];
        if (s == 0.f) continue;
        int2 ij = g.edges[e];
        const float* a = g.in1 + size_t(g.loc1[ij.x]) * g.w1;
        const float* b = g.in2 + size_t(g.loc2[ij.y]) * g.w2;
        int t1 = g.type1[ij.x], t2 = g.type2[ij.y];
        const float* p = g.param + (size_t(t1) * g.n_type2 + t2) * g.n_param;
        int n_ka = 15, n_k = g.kind == IK_ROTAMER ? 12 : 10;
        float inv_dx = g.kind == IK_ROTAMER ? 1.f / 0.7f : 1.f / 0.625f;
        float pre = 1.f;
        if (g.kind == IK_HBCOV) pre = (1.f - a[6]) * (1.f - a[6]);
        f3 disp = min_image(ld3(b) - ld3(a), g.box), r1 = ld3(a + 3), r2 = ld3(b + 3);
        float dist2 = mag2(disp), inv_dist = rsqrtf(dist2);
        float dc = dist2 * (inv_dist * inv_dx);
        f3 u = disp * inv_dist;
        float x1s = (dot(r1, u) + 1.f) * 6.f + 1.f, x2s = (-dot(r2, u) + 1.f) * 6.f + 1.f;
        float a1v, a1d, a2v, a2d, nv, nd, r[4];
        deboor(p, x1s, a1v, a1d);
        deboor(p + n_ka, x2s, a2v, a2d);
        clamped(p + 2 * n_ka + n_k, dc, n_k, nv, nd);
        float w = s * pre;
        float* o1 = out + (size_t(t1) * g.n_type2 + t2) * g.n_param;
        float* o2 = out + (size_t(t2) * g.n_type1 + t1) * g.n_param;
        int sb = clamped_coeff_deriv(dc, n_k, r);
        for (int i = 0; i < 4; ++i) {
            atomicAdd(o1 + 2 * n_ka + sb + i, w * r[i]);
            atomicAdd(o1 + 2 * n_ka + n_k + sb + i, w * a1v * a2v * r[i]);
            if (g.symmetric) {
                atomicAdd(o2 + 2 * n_ka + sb + i, w * r[i]);
                atomicAdd(o2 + 2 * n_ka + n_k + sb + i, w * a1v * a2v * r[i]);
            }
        }
        sb = coeff_deriv(x1s, r);
        for (int i = 0; i < 4; ++i) {
            atomicAdd(o1 + sb + i, w * a2v * nv * r[i]);
            if (g.symmetric) atomicAdd(o2 + sb + i, w * a2v * nv * r[i]);
        }
        sb = coeff_deriv(x2s, r);
        for (int i = 0; i < 4; ++i) {
            atomicAdd(o1 + n_ka + sb + i, w * a1v * nv * r[i]);
            if (g.symmetric) atomicAdd(o2 + n_ka + sb + i, w * a1v * nv * r[i]);
        }
    }
}

void launch_param_deriv(const DGraph& g, float* out, cudaStream_t st) {
    ug::launch(param_deriv_kernel, 2 * 152, 256, 0, st, g, out);
}

// ------------------------------------------------------------ rotamer BP ---
__device__ __forceinline__ long long slot_index(const DBP& b, int r1, int r2) {
    int s = b.res_sys[r1];
    return b.slot_off[s] + (long long)b.res_local[r1] * b.res_N[r1] + b.res_local[r2];
}

// reset the residue-pair map entries of the previous evaluation and the
// per-residue accumulators
__global__ void bp_reset_kernel(DBP b) {
    grid_dep_entry();
    int prev_n_ent = min(*b.n_ent, b.ent_cap);  // entries of the previous evaluation
    for (int e = grid_stride_start(); e < prev_n_ent; e += grid_stride())
        b.slot[slot_index(b, b.erow[e], b.col[e])] = -1;
    for (int r = grid_stride_start(); r < b.n_res * 8; r += grid_stride()) {
        b.E1[r] = 0.f;
        b.E1x[r] = 0.f;
    }
    for (int s = grid_stride_start(); s < b.n_sys; s += grid_stride()) b.e11[s] = 0.0;
    for (int r = grid_stride_start(); r < b.n_res; r += grid_stride()) b.row_count[r] = 0;
    if (b.reuse && blockIdx.x == 0 && threadIdx.x == 0) *b.parity ^= 1;  // new evaluation
}

// 1-body energy per (residue, rotamer) from up to 4 input nodes (src/rotamer.cpp:862-884)
__global__ void bp_bead_energy_kernel(DBP b, const float* p0, const float* p1, const float* p2, const float* p3,
                                      int n_in, int w0, int w1, int w2, int w3) {
    grid_dep_entry();
    for (int i = grid_stride_start(); i < b.n_bead; i += grid_stride()) {
        int l = b.bead_loc[i];
        float e = p0[size_t(l) * w0];
        if (n_in > 1) e += p1[size_t(l) * w1];
        if (n_in > 2) e += p2[size_t(l) * w2];
        if (n_in > 3) e += p3[size_t(l) * w3];
        atomicAdd(&b.E1[b.bead_res[i] * 8 + b.bead_rot[i]], e);
    }
}

// The rotamer graph's edge values and derivatives (edge_eval_kernel) and, from
// each value at once, the classification of the bead edges: multi-rotamer
// residue pairs marked in the dense map, 1-rotamer partners folded into node
// energies, 1-1 edges summed (src/rotamer.cpp:886-912).  The slot reset
// (bp_reset_kernel) runs before the pair search.
__global__ void rotamer_edge_kernel(DGraph g, DBP b) {
    grid_dep_entry();
    const int ne = *g.n_edge;
    const int dw = g.d1 + g.d2;
    for (int e = grid_stride_start(); e < ne; e += grid_stride()) {
        const int2 ij = g.edges[e];
        const float* pa = g.in1 + size_t(g.loc1[ij.x]) * g.w1;
        const float* pb = g.in2 + size_t(g.loc2[ij.y]) * g.w2;
        const float* p = g.param + (size_t(g.type1[ij.x]) * g.n_type2 + g.type2[ij.y]) * g.n_param;
        float* da = g.deriv + size_t(e) * dw;
        const float v = edge_value<IK_ROTAMER>(g, p, pa, pb, da, da + g.d1, true);
        g.value[e] = v;
        const int r1 = b.bead_res[ij.x], r2 = b.bead_res[ij.y];
        const int n1 = b.nrot[r1], n2 = b.nrot[r2];
        if (n1 > 1 && n2 > 1) {
            // each residue pair counts once in both rows' entry counts
            if (atomicExch(&b.slot[slot_index(b, r1, r2)], -2) != -2) atomicAdd(&b.row_count[r1], 1);
            if (atomicExch(&b.slot[slot_index(b, r2, r1)], -2) != -2) atomicAdd(&b.row_count[r2], 1);
        } else if (n1 == 1 && n2 == 1) {
            atomicAdd(&b.e11[b.res_sys[r1]], double(v));
            if (b.log_e11) {
                atomicAdd(&b.log_e11[r1], 0.5f * v);
                atomicAdd(&b.log_e11[r2], 0.5f * v);
            }
        } else if (n1 == 1) {
            atomicAdd(&b.E1x[r2 * 8 + b.bead_rot[ij.y]], v);
        } else {
            atomicAdd(&b.E1x[r1 * 8 + b.bead_rot[ij.x]], v);
        }
    }
}

// warp per residue row of the dense map: emit the marked neighbours in
// increasing order at the row's scanned offset (the rows' counts come from the
// marking, rotamer_edge_kernel)
__global__ void bp_rows_kernel(DBP b) {
    grid_dep_entry();
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    int n_warps = (gridDim.x * blockDim.x) >> 5;
    for (int r = warp; r < b.n_res; r += n_warps) {
        int N = b.res_N[r];
        int s = b.res_sys[r];
        int rbase = b.res_off[s];
        long long row = b.slot_off[s] + (long long)b.res_local[r] * N;
        int pos = b.row_ptr[r];
        // the row's slots are read a batch of ROWS_BATCH x 32 at a time, all
        // loads in flight together, before any of them is rewritten (only
        // this warp touches the row)
        constexpr int ROWS_BATCH = 16;
        for (int c00 = 0; c00 < N; c00 += 32 * ROWS_BATCH) {
            int v[ROWS_BATCH];
#pragma unroll
            for (int k = 0; k < ROWS_BATCH; ++k) {
                const int c = c00 + 32 * k + lane;
                v[k] = c < N ? b.slot[row + c] : -1;
            }
#pragma unroll
            for (int k = 0; k < ROWS_BATCH; ++k) {
                const int c = c00 + 32 * k + lane;
                const bool hit = v[k] == -2;  // c < N
                unsigned m = __ballot_sync(0xffffffffu, hit);
                if (hit) {
                    int p = pos + __popc(m & ((1u << lane) - 1u));
                    if (p < b.ent_cap) {
                        b.col[p] = rbase + c;
                        b.erow[p] = r;
                        b.slot[row + c] = p;
                        float4* z = reinterpret_cast<float4*>(b.esum + size_t(p) * 36);  // summed below
#pragma unroll
                        for (int q = 0; q < 9; ++q) z[q] = make_float4(0.f, 0.f, 0.f, 0.f);
                    } else {
                        b.slot[row + c] = -1;
                    }
                }
                pos += __popc(m);
            }
        }
    }
}

// Summed pair energies of the entries; and per bead edge, where the
// sensitivity pass finds the edge's weight (eaux): an edge-marginal element
// (>= 0), 1 for two single-rotamer beads (BP_W_ONE), the node marginal of the
// multi-rotamer partner (BP_W_NODE - index), or none (BP_W_NONE, entry lost to
// overflow)
#define BP_W_ONE (-1)
#define BP_W_NODE (-2)
#define BP_W_NONE INT_MIN
// The same kernel completes the entries (reverse entry and descriptor; a
// partner entry lost to overflow points at itself and is flagged); the
// entries' energy sums were zeroed as the rows emitted them.
__global__ void bp_edge_energy_kernel(DBP b, DGraph g) {
    grid_dep_entry();
    const int n = min(*b.n_ent, b.ent_cap);
    for (int e = grid_stride_start(); e < n; e += grid_stride()) {
        int rv = b.slot[slot_index(b, b.col[e], b.erow[e])];
        if (rv < 0) {
            atomicOr(b.status, ST_RES_EDGE_OVERFLOW);
            rv = e;
        }
        b.rev[e] = rv;
        b.einfo[e] = make_int4(b.res_local[b.erow[e]], rv, b.res_local[b.col[e]], 0);
    }
    int ne = *g.n_edge;
    for (int e = grid_stride_start(); e < ne; e += grid_stride()) {
        int2 ij = g.edges[e];
        int r1 = b.bead_res[ij.x], r2 = b.bead_res[ij.y];
        int n1 = b.nrot[r1], n2 = b.nrot[r2];
        int k1 = b.bead_rot[ij.x], k2 = b.bead_rot[ij.y];
        if (n1 == 1 || n2 == 1) {
            g.eaux[e] = n1 == 1 && n2 == 1 ? BP_W_ONE : BP_W_NODE - (n1 == 1 ? r2 * 8 + k2 : r1 * 8 + k1);
            continue;
        }
        int e12 = b.slot[slot_index(b, r1, r2)], e21 = b.slot[slot_index(b, r2, r1)];
        g.eaux[e] = e12 >= 0 ? e12 * 36 + k1 * 6 + k2 : BP_W_NONE;
        if (e12 < 0 || e21 < 0) continue;
        float v = g.value[e];
        atomicAdd(&b.esum[size_t(e12) * 36 + k1 * 6 + k2], v);
        atomicAdd(&b.esum[size_t(e21) * 36 + k2 * 6 + k1], v);
    }
}

// One-body energies and node probabilities in one pass (beads grouped by
// residue): each residue's beads summed in bead order, as the reference fills
// its node holders (src/rotamer.cpp:862-884), then bp_node_prob_kernel's
// probabilities
__global__ void bp_bead_prob_kernel(DBP b, const float* p0, const float* p1, const float* p2, const float* p3,
                                    int n_in, int w0, int w1, int w2, int w3) {
    grid_dep_entry();
    for (int r = grid_stride_start(); r < b.n_res; r += grid_stride()) {
        float E[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) E[k] = 0.f;
        for (int i = b.res_bead_off[r]; i < b.res_bead_off[r + 1]; ++i) {
            const int l = b.bead_loc[i];
            float e = p0[size_t(l) * w0];
            if (n_in > 1) e += p1[size_t(l) * w1];
            if (n_in > 2) e += p2[size_t(l) * w2];
            if (n_in > 3) e += p3[size_t(l) * w3];
            const int k = b.bead_rot[i];
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (q == k) E[q] += e;
        }
        const int n = b.nrot[r];
#pragma unroll
        for (int k = 0; k < 8; ++k) b.E1[r * 8 + k] = E[k];
        float m = E[0];
#pragma unroll
        for (int k = 1; k < 8; ++k)
            if (k < n) m = fminf(m, E[k]);
#pragma unroll
        for (int k = 0; k < 8; ++k) b.prob[r * 8 + k] = k < n ? expf(m - E[k]) * expf(-b.E1x[r * 8 + k]) : 0.f;
        b.eoff[r] = m;
    }
}

// node probabilities (src/rotamer.cpp:239-256, :398-405)
__global__ void bp_node_prob_kernel(DBP b) {
    grid_dep_entry();
    for (int r = grid_stride_start(); r < b.n_res; r += grid_stride()) {
        int n = b.nrot[r];
        float m = b.E1[r * 8];
        for (int k = 1; k < n; ++k) m = fminf(m, b.E1[r * 8 + k]);
        for (int k = 0; k < 8; ++k)
            b.prob[r * 8 + k] = k < n ? expf(m - b.E1[r * 8 + k]) * expf(-b.E1x[r * 8 + k]) : 0.f;
        b.eoff[r] = m;
    }
}
// pair probability matrices from the summed pair energies alone (they need no
// one-body energy): one thread per entry, its 6x6 block as nine float4, zero
// outside the (row rotamers) x (column rotamers) corner
__global__ void bp_pair_prob_kernel(DBP b) {
    grid_dep_entry();
    int n_ent = min(*b.n_ent, b.ent_cap);
    for (int e = grid_stride_start(); e < n_ent; e += grid_stride()) {
        int nu = b.nrot[b.erow[e]], nv = b.nrot[b.col[e]];
        const float4* src = reinterpret_cast<const float4*>(b.esum + size_t(e) * 36);
        float4* dst = reinterpret_cast<float4*>(b.P + size_t(e) * 36);
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            float4 x = src[q];
            float v[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                int k = 4 * q + j, a = k / 6, c = k - a * 6;
                v[j] = (a < nu && c < nv) ? expf(-v[j]) : 0.f;
            }
            dst[q] = make_float4(v[0], v[1], v[2], v[3]);
        }
    }
}

// ---------------------------------------------------------------------------
// BP solve.  One block per system.  A sweep has two phases separated by a
// block barrier:
//   messages: one thread per directed entry f = (v <- u) of the system.  From
//     v's old belief divided by the old message into v along f, and f's
//     matrix P_f(x_v, x_u), it forms the new message from v to u and stores
//     it in the reverse entry (u <- v), the slot u reads;
//   beliefs: one thread per node u multiplies its incoming new messages into
//     prob_u and applies the reference's normalisation, damping and
//     one-sided deviation.
// This is the reference's Jacobi sweep (every read from the old buffers)
// with the message computed by the sending node, so each thread's loads are
// independent of the others'.  The iteration structure (undamped first sweep
// with swap, chunks of `chunk` damped sweeps, one-sided maximum deviation
// test) follows src/rotamer.cpp:1106-1162; the messages and beliefs follow
// src/rotamer.cpp:259-281, :500-569; the marginals and Bethe free energy
// src/rotamer.cpp:425-471.  Node beliefs (both buffers) and rotamer counts
// live in shared memory; P and messages stay in global memory (L2-resident).
// Division in the sweeps is multiplication by a reciprocal from the special
// function unit (__fdividef, about 2 ulp), as the reference multiplies by its
// approximate reciprocal refined once (rcp, src/Float4.h:225-238).
__device__ __forceinline__ void renorm6(float* x, int n) {
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 6; ++k) s += k < n ? x[k] : 0.f;
    float inv = __fdividef(1.f, s);
#pragma unroll
    for (int k = 0; k < 6; ++k) x[k] *= inv;
}
// Exact rescaling of a non-negative product by a power of two so that its
// largest entry lies in [1, 2): keeps a running product of messages (each
// summing to 1) away from underflow without a division or any rounding.
__device__ __forceinline__ void rescale6(float* x) {
    float m = fmaxf(fmaxf(fmaxf(x[0], x[1]), fmaxf(x[2], x[3])), fmaxf(x[4], x[5]));
    const int e = (__float_as_int(m) >> 23) & 0xff;
    if (e >= 1 && e <= 253) {
        const float sc = __int_as_float((254 - e) << 23);  // 2^(127 - e)
#pragma unroll
        for (int k = 0; k < 6; ++k) x[k] *= sc;
    }
}

// Where the solve's two message buffers live.  Global: b.msg + k ent_cap 8
// + 8 e for every entry e of the batch.  Shared (dsm): each block holds both
// buffers for its own entries [base, base + dsm_cap) in its shared memory
// from s0 (buffer 0, buffer 1, then the destination table: own entry
// f - base -> (owner rank << 20) | slot of rev(f) in the owner), and a sender
// stores a message straight into the shared memory of the block that owns
// the entry it writes (distributed shared memory).  Both phases then read
// only local shared memory; the cluster barrier between them orders the
// stores.  Global buffers and sizes are read from the kernel parameters.
struct MsgLoc {
    float* s0;
    int base;
    int dsm;
    __device__ __forceinline__ float* shared(const DBP& b, int k) const {
        return s0 + (k ? size_t(b.dsm_cap) * 8 : 0);
    }
    __device__ __forceinline__ int* dst_table(const DBP& b) const {
        return reinterpret_cast<int*>(s0 + size_t(b.dsm_cap) * 16);
    }
    __device__ __forceinline__ float* own(const DBP& b, int k, int e) const {
        return dsm ? shared(b, k) + size_t(e - base) * 8 : b.msg + (k ? size_t(b.ent_cap) * 8 : 0) + size_t(e) * 8;
    }
};

// Per-sweep constants of a block's own share in shared memory (compact layout
// whose cluster fits): per own entry its row and column nodes (system-local),
// per own node its prob row and first entry (clipped to the system's end).
// When ok is false the sweeps read them from global memory.
struct BpOwn {
    int *row = nullptr, *col = nullptr, *rp = nullptr;
    float* prob = nullptr;
    bool ok = false;
};

// new message along every entry of [e0, e1): einfo[f] = (local index of the
// row node v, reverse entry, local index of the column node u, 0); the old
// message is read from buffer kold, the new one written to buffer kcur.
// Beliefs are indexed from node nb_lo.
__device__ __forceinline__ void bp_messages(const DBP& b, int e0, int e1, const float* __restrict__ Nold, int nb_lo,
                                            const int* __restrict__ s_nrot, const MsgLoc& M, const BpOwn& OW,
                                            int kold, int kcur, cg::cluster_group& cluster, int tid, int nt) {
    for (int f = e0 + tid; f < e1; f += nt) {
        int4 inf;
        if (OW.ok) {
            inf.x = OW.row[f - e0];
            inf.z = OW.col[f - e0];
            inf.y = 0;  // the destination table gives the reverse entry's slot
        } else {
            inf = b.einfo[f];
        }
        int nv = s_nrot[inf.x], nu = s_nrot[inf.z];
        const float* ob = Nold + (inf.x - nb_lo) * 8;
        const float4* om = reinterpret_cast<const float4*>(M.own(b, kold, f));
        float4 o0 = om[0], o1 = om[1];
        float omv[6] = {o0.x, o0.y, o0.z, o0.w, o1.x, o1.y};
        float cav[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) cav[k] = k < nv ? __fdividef(ob[k], 1e-10f + omv[k]) : 0.f;
        const float4* P4 = reinterpret_cast<const float4*>(b.P + size_t(f) * 36);
        float P[36];
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            float4 t = __ldg(P4 + q);
            P[4 * q] = t.x; P[4 * q + 1] = t.y; P[4 * q + 2] = t.z; P[4 * q + 3] = t.w;
        }
        float mm[6], sum = 0.f;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            float acc = 0.f;
#pragma unroll
            for (int k = 0; k < 6; ++k) acc += P[k * 6 + i] * cav[k];
            mm[i] = i < nu ? acc : 0.f;
            sum += mm[i];
        }
        float inv = __fdividef(1.f, sum);
        float4* out;
        if (M.dsm) {
            int d = M.dst_table(b)[f - M.base];
            out = reinterpret_cast<float4*>(cluster.map_shared_rank(M.shared(b, kcur) + size_t(d & 0xFFFFF) * 8, d >> 20));
        } else {
            out = reinterpret_cast<float4*>(b.msg + (kcur ? size_t(b.ent_cap) * 8 : 0) + size_t(inf.y) * 8);
        }
        out[0] = make_float4(mm[0] * inv, mm[1] * inv, mm[2] * inv, mm[3] * inv);
        out[1] = make_float4(mm[4] * inv, mm[5] * inv, 0.f, 0.f);
    }
}

// new beliefs of nodes [lo, hi); returns this thread's largest one-sided
// deviation (mode 1).  BP_LANES consecutive lanes share a node: each folds
// every BP_LANES-th incoming message, then the partial products are combined
// across the group with shuffles, so a node's latency chain is its degree /
// BP_LANES loads.
template <int BP_LANES>
__device__ __forceinline__ float bp_beliefs(const DBP& b, int r0, int lo, int hi, int e1, const float* __restrict__ Nold,
                                            float* __restrict__ Ncur, int nb_lo, const int* __restrict__ s_nrot,
                                            const MsgLoc& M, const BpOwn& OW, int kcur, int mode, float damp, int tid,
                                            int nt) {
    float dev = 0.f;
    const int q = tid % BP_LANES, lane = tid & 31;
    const unsigned gmask = ((1u << BP_LANES) - 1u) << (lane & ~(BP_LANES - 1));
    auto m4 = [&](int e) { return reinterpret_cast<const float4*>(M.own(b, kcur, e)); };
    for (int ul = lo + tid / BP_LANES; ul < hi; ul += nt / BP_LANES) {  // group-uniform
        int n = s_nrot[ul];
        if (n == 1) continue;
        int u = r0 + ul;
        int eb = OW.ok ? OW.rp[ul - lo] : b.row_ptr[u], ee = OW.ok ? OW.rp[ul - lo + 1] : min(b.row_ptr[u + 1], e1);
        float prod[6] = {1.f, 1.f, 1.f, 1.f, 1.f, 1.f};
        // rescaled by a power of two after every factor, so the product never
        // underflows (each message sums to 1); the sum normalisation of the
        // reference's running product (src/rotamer.cpp:538-539) is applied
        // once, to the finished belief below: the scale cancels there
        auto fold = [&](const float* a) {
#pragma unroll
            for (int k = 0; k < 6; ++k) prod[k] *= a[k];
            rescale6(prod);
        };
        int e = eb + q;
        for (; e + BP_LANES < ee; e += 2 * BP_LANES) {  // two loads in flight
            const float4 *p0 = m4(e), *p1 = m4(e + BP_LANES);
            float4 a0 = p0[0], c0 = p0[1];
            float4 a1 = p1[0], c1 = p1[1];
            float x0[6] = {a0.x, a0.y, a0.z, a0.w, c0.x, c0.y}, x1[6] = {a1.x, a1.y, a1.z, a1.w, c1.x, c1.y};
            fold(x0);
            fold(x1);
        }
        if (e < ee) {
            const float4* p0 = m4(e);
            float4 a0 = p0[0], c0 = p0[1];
            float x0[6] = {a0.x, a0.y, a0.z, a0.w, c0.x, c0.y};
            fold(x0);
        }
#pragma unroll
        for (int o = BP_LANES / 2; o > 0; o >>= 1) {
            float y[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) y[k] = __shfl_xor_sync(gmask, prod[k], o);
            fold(y);
        }
        if (q != 0) continue;
        float bl[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) bl[k] = k < n ? (OW.ok ? OW.prob[(ul - lo) * 8 + k] : b.prob[u * 8 + k]) * prod[k] : 0.f;
        renorm6(bl, n);
        const float* o = Nold + (ul - nb_lo) * 8;
        if (mode == 1) {
            float mx = bl[0];
            for (int k = 1; k < n; ++k) mx = fmaxf(mx, bl[k]);
            float inv = __fdividef(1.f, mx);
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                bl[k] = damp != 0.f ? (1.f - damp) * inv * bl[k] + damp * o[k] : inv * bl[k];
                if (k < n) dev = fmaxf(dev, bl[k] - o[k]);
            }
        }
        float* c = Ncur + (ul - nb_lo) * 8;
#pragma unroll
        for (int k = 0; k < 6; ++k) c[k] = bl[k];
        c[6] = c[7] = 0.f;
    }
    return dev;
}

// One cluster of BP_CLUSTER blocks per system.  Block c of the cluster owns a
// contiguous range of the system's nodes, split so that every block gets
// about the same number of directed entries (the CSR rows of its nodes), and
// runs both phases over its own entries and nodes.  Messages cross blocks
// through global memory: a block writes the reverse entries of its rows, and
// the cluster barrier between the phases (release/acquire at cluster scope)
// makes them visible to their owners.  Beliefs never leave their block.
// Template: BP_CLUSTER blocks (SMs) per system, BP_LANES lanes per node in
// the belief phase, THREADS threads per block; the variants are listed in
// bp_variants (the engine's autotuner picks one).
template <int BP_CLUSTER, int BP_LANES, int THREADS>
__global__ void __launch_bounds__(THREADS, 65536 / (THREADS * 64)) bp_solve_kernel(DBP b, int want_energy, double* energy_out) {
    grid_dep_entry();
    extern __shared__ float smem[];
    __shared__ double dred[32];
    __shared__ float s_dev[2][BP_CLUSTER];  // per chunk parity: every block's deviation maximum
    __shared__ int s_bmax[2];               // this block's maximum (non-negative float bits)
    __shared__ double s_en[BP_CLUSTER];
    cg::cluster_group cluster = cg::this_cluster();
    const int crank = int(cluster.block_rank());
    const int s = blockIdx.x / BP_CLUSTER;
    const int r0 = b.res_off[s], r1 = b.res_off[s + 1], N = r1 - r0;
    const int e0 = b.row_ptr[r0], e1 = min(b.row_ptr[r1], b.ent_cap);
    const bool compact = b.dsm_cap > 0;
    // the system's row starts, staged in shared memory for the block splits
    // (binary searches there instead of chains of dependent global loads);
    // the layout below overwrites the staging area after the splits
    int* s_rp = reinterpret_cast<int*>(compact ? smem + ((N + 3) & ~3) : smem);
    for (int i = threadIdx.x; i <= N; i += blockDim.x) s_rp[i] = b.row_ptr[r0 + i];
    __syncthreads();
    // own nodes [lo, hi) (system-local): block c starts at the first node whose
    // row begins at or after c/BP_CLUSTER of the system's entries
    auto split = [&](int c) -> int {
        if (c <= 0) return 0;
        if (c >= BP_CLUSTER) return N;
        long long target = e0 + (long long)(e1 - e0) * c / BP_CLUSTER;
        int a = 0, z = N;  // first ul in [0, N] with row_ptr[r0 + ul] >= target
        while (a < z) {
            int m = (a + z) >> 1;
            if (s_rp[m] >= target) z = m; else a = m + 1;
        }
        return a;
    };
    const int lo = split(crank), hi = split(crank + 1);
    const int eo0 = min(s_rp[lo], e1), eo1 = min(s_rp[hi], e1);
    float* EM[2] = {b.msg, b.msg + size_t(b.ent_cap) * 8};
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;

    // Shared layout.  Full (dsm_cap 0): beliefs of all N nodes (both
    // buffers), then the rotamer counts; messages in global memory.  Compact
    // (dsm_cap > 0): rotamer counts of all N nodes, beliefs of the block's own
    // nodes (nb_cap per buffer), then both message buffers of its own entries
    // (dsm_cap slots each) and the destination table.  Compact is used when
    // every block of the cluster fits (each block computes every block's
    // ranges, so the decision is the same in all); otherwise the own beliefs
    // go to the global scratch and the messages to global memory.
    __shared__ int s_eb[BP_CLUSTER + 1], s_nb[BP_CLUSTER + 1];
    if (tid <= BP_CLUSTER) {
        int sp = split(tid);
        s_nb[tid] = sp;
        s_eb[tid] = min(s_rp[sp], e1);
    }
    __syncthreads();
    bool fits = compact;
    for (int c = 0; c < BP_CLUSTER; ++c)
        if (s_eb[c + 1] - s_eb[c] > b.dsm_cap || s_nb[c + 1] - s_nb[c] > b.nb_cap) fits = false;
    float* NB[2];
    int* s_nrot;
    int nb_lo = 0;
    BpOwn OW;
    MsgLoc M;
    M.base = eo0;
    M.dsm = fits;
    M.s0 = nullptr;
    if (!compact) {
        NB[0] = smem;
        NB[1] = smem + N * 8;
        s_nrot = reinterpret_cast<int*>(smem + 2 * N * 8);
    } else {
        s_nrot = reinterpret_cast<int*>(smem);
        float* nbb = smem + ((N + 3) & ~3);
        nb_lo = lo;
        if (fits) {
            NB[0] = nbb;
            NB[1] = nbb + size_t(b.nb_cap) * 8;
        } else {
            NB[0] = b.nb_scratch + size_t(r0 + lo) * 8;
            NB[1] = b.nb_scratch + (size_t(b.n_res) + r0 + lo) * 8;
        }
        M.s0 = nbb + size_t(b.nb_cap) * 16;
        // after the destination table, the per-sweep constants of the
        // block's share: own nodes' prob rows and first entries, own entries'
        // row and column nodes, so that a sweep reads only shared memory and P
        OW.prob = M.s0 + size_t(b.dsm_cap) * 17;
        OW.rp = reinterpret_cast<int*>(OW.prob + size_t(b.nb_cap) * 8);
        OW.row = OW.rp + b.nb_cap + 1;
        OW.col = OW.row + b.dsm_cap;
        OW.ok = fits;
        if (fits) {
            int* dst = M.dst_table(b);
            for (int f = eo0 + tid; f < eo1; f += nt) {
                int rv = b.rev[f];  // same system: within [s_eb[0], s_eb[BP_CLUSTER])
                int c = 0;
                while (c + 1 < BP_CLUSTER && rv >= s_eb[c + 1]) ++c;
                dst[f - eo0] = (c << 20) | (rv - s_eb[c]);
                const int4 inf = b.einfo[f];
                OW.row[f - eo0] = inf.x;
                OW.col[f - eo0] = inf.z;
            }
            for (int li = tid; li < hi - lo; li += nt) {
                const float4* pr = reinterpret_cast<const float4*>(b.prob + size_t(r0 + lo + li) * 8);
                reinterpret_cast<float4*>(OW.prob)[2 * li] = pr[0];
                reinterpret_cast<float4*>(OW.prob)[2 * li + 1] = pr[1];
            }
            for (int li = tid; li <= hi - lo; li += nt) OW.rp[li] = min(b.row_ptr[r0 + lo + li], e1);
        }
    }

    auto sweep = [&](const float* Nold, float* Ncur, int kold, int kcur, int mode, float damp) {
        bp_messages(b, eo0, eo1, Nold, nb_lo, s_nrot, M, OW, kold, kcur, cluster, tid, nt);
        cluster.sync();
        return bp_beliefs<BP_LANES>(b, r0, lo, hi, e1, Nold, Ncur, nb_lo, s_nrot, M, OW, kcur, mode, damp, tid, nt);
    };
    if (tid < 2) s_bmax[tid] = 0;

    // Learned warm start: the first sweep starts from the predicted marginals
    // instead of prob.  Per system, the mean sweep counts of warm and uniform
    // starts are tracked (warm_stat: mean warm, mean uniform, solves); every
    // WARM_PROBE-th solve tries the other start to refresh the comparison,
    // and the warm start is used only while it saves WARM_MIN_GAIN sweeps
    // (warm_start_used).
    const int par = b.reuse ? *b.parity : 0;
    const bool use_prev = b.reuse && b.prev_valid[(par ^ 1) * b.n_sys + s];
    const bool use_warm = use_prev || (b.warm && warm_start_used(b.warm_stat + 4 * s, b.warm_gain));
    const float* init = use_prev ? b.marg : use_warm ? b.warm : b.prob;
    // N.old = N.cur = prob (N.old = prediction when warm); E.old = 1 (own entries)
    for (int ul = tid; ul < N; ul += nt) s_nrot[ul] = b.nrot[r0 + ul];
    for (int ul = lo + tid; ul < hi; ul += nt) {  // own nodes
        // a start row that is not a distribution (no previous solve yet) falls
        // back to prob for that node
        const float* w = init + (r0 + ul) * 8;
        float ws = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) ws += w[k];
        if (!(ws > 0.5f)) w = b.prob + (r0 + ul) * 8;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            NB[0][(ul - nb_lo) * 8 + k] = b.prob[(r0 + ul) * 8 + k];
            NB[1][(ul - nb_lo) * 8 + k] = w[k];
        }
    }
    __syncthreads();
    if (use_prev) {
        // the previous solve's final message of the same residue pair (u <- v),
        // found in u's previous CSR row (columns ascending); uniform if the
        // pair is new
        const int q = par ^ 1;
        const int* pr = b.prev_row_ptr + size_t(q) * (b.n_res + 1);
        const int* pc = b.prev_col + size_t(q) * b.ent_cap;
        const float* pm = b.prev_msg + size_t(q) * b.ent_cap * 8;
        for (int f = eo0 + tid; f < eo1; f += nt) {
            int u = b.erow[f], v = b.col[f];
            int a = pr[u], z = pr[u + 1];
            while (a < z) {  // first previous column >= v
                int m = (a + z) >> 1;
                if (pc[m] < v) a = m + 1; else z = m;
            }
            float4* dst = reinterpret_cast<float4*>(M.own(b, 1, f));
            if (a < pr[u + 1] && pc[a] == v) {
                const float4* src = reinterpret_cast<const float4*>(pm + size_t(a) * 8);
                dst[0] = src[0];
                dst[1] = src[1];
            } else {
                dst[0] = dst[1] = make_float4(1.f, 1.f, 1.f, 1.f);
            }
        }
    } else if (!use_warm) {
        float* m1 = M.own(b, 1, eo0);  // own entries are contiguous in either place
        for (int i = tid; i < (eo1 - eo0) * 8; i += nt) m1[i] = 1.f;
    } else {
        // messages consistent with the start: the d incoming messages of node
        // u are all (start_u / prob_u)^(1/d), so that prob_u times their
        // product is the start belief
        for (int f = eo0 + tid; f < eo1; f += nt) {
            int u = b.erow[f], ul = u - r0;
            int n = s_nrot[ul];
            float inv_d = 1.f / float(max(1, b.row_ptr[u + 1] - b.row_ptr[u]));
            float m[8], sum = 0.f;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                m[k] = k < n ? powf((1e-10f + NB[1][(ul - nb_lo) * 8 + k]) / (1e-10f + NB[0][(ul - nb_lo) * 8 + k]), inv_d)
                             : 0.f;
                sum += m[k];
            }
            float inv = 1.f / sum;
            float* mf = M.own(b, 1, f);
#pragma unroll
            for (int k = 0; k < 8; ++k) mf[k] = k < n ? m[k] * inv : 1.f;
        }
    }
    __syncthreads();
    const int chunk = max(1, b.chunk);
    int nc = 1, ec = 0;
    float dev = 1e10f;
    int iter = 0;
    // first sweep, undamped: new beliefs go to the buffer that then becomes
    // "old"; the other (prob) is max-normalised (src/rotamer.cpp:1135)
    if (M.dsm) cluster.sync();  // every block of the cluster runs before shared stores reach it
    sweep(NB[1], NB[0], 1, 0, 0, 0.f);
    __syncthreads();
    for (int ul = lo + tid; ul < hi; ul += nt) {
        int n = s_nrot[ul];
        if (n == 1) continue;
        float* c = NB[1] + (ul - nb_lo) * 8;
        float mx = c[0];
        for (int k = 1; k < n; ++k) mx = fmaxf(mx, c[k]);
        float inv = 1.f / mx;
        for (int k = 0; k < 6; ++k) c[k] *= inv;
    }
    __syncthreads();
    // Chunks of damped sweeps until the largest one-sided deviation of a
    // chunk's last sweep is within tol (src/rotamer.cpp:1137-1156).  The
    // cluster-wide maximum needs no barrier of its own: each block posts its
    // maximum into slot crank of every block (parity cpar), and the slots are
    // read after the next sweep's message-phase barrier.  When they say
    // "converged", that message phase (written into the older message buffer,
    // which nothing reads afterwards) is discarded and the state is the one
    // after the converged chunk: the same sweeps and results as a separate
    // barrier before every test.
    int cpar = 0;
    bool pending = false;
    while (iter < b.max_iter) {
        float d = 0.f;
        bool converged = false;
        for (int j = 0; j < chunk; ++j) {
            nc ^= 1;
            ec ^= 1;
            bp_messages(b, eo0, eo1, NB[nc ^ 1], nb_lo, s_nrot, M, OW, ec ^ 1, ec, cluster, tid, nt);
            cluster.sync();
            if (pending) {  // the previous chunk's maximum, posted before this barrier
                pending = false;
                float r = 0.f;
#pragma unroll
                for (int c = 0; c < BP_CLUSTER; ++c) r = fmaxf(r, s_dev[cpar ^ 1][c]);
                dev = r;
                if (!(dev > b.tol)) {
                    nc ^= 1;
                    ec ^= 1;
                    converged = true;
                    break;
                }
            }
            d = bp_beliefs<BP_LANES>(b, r0, lo, hi, e1, NB[nc ^ 1], NB[nc], nb_lo, s_nrot, M, OW, ec, 1, b.damping, tid,
                                     nt);
            if (j == chunk - 1) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) d = fmaxf(d, __shfl_xor_sync(0xffffffffu, d, o));
                if (lane == 0) atomicMax(&s_bmax[cpar], __float_as_int(d));  // d >= 0
            }
            __syncthreads();
        }
        if (converged) break;
        iter += chunk;
        if (tid < BP_CLUSTER) *cluster.map_shared_rank(&s_dev[cpar][crank], tid) = __int_as_float(s_bmax[cpar]);
        if (tid == 0) s_bmax[cpar ^ 1] = 0;
        cpar ^= 1;
        pending = true;
    }
    if (M.dsm) {  // final messages of own entries to global memory, for the tail and later kernels
        const float4* src = reinterpret_cast<const float4*>(M.shared(b, ec));
        float4* dstg = reinterpret_cast<float4*>(EM[ec] + size_t(eo0) * 8);
        for (int i = tid; i < (eo1 - eo0) * 2; i += nt) dstg[i] = src[i];
        __syncthreads();
    }
    if (tid == 0 && crank == 0) {
        b.n_iter[s] = iter;
        if (iter >= b.max_iter - b.chunk - 1) {
            atomicOr(b.status, ST_BP_NOT_CONVERGED);
            if (b.bad_solves) b.bad_solves[s] += 1ull;
        }
        if (b.warm) {  // running means of the sweep counts of both starts
            float* ws = b.warm_stat + 4 * s;
            float sweeps = float(1 + iter);
            int k = use_warm ? 0 : 1, known = int(ws[3]);
            ws[k] = (known >> k & 1) ? 0.75f * ws[k] + 0.25f * sweeps : sweeps;
            ws[2] += 1.f;
            ws[3] = float(known | (1 << k));
        }
    }
    // node marginals of own nodes
    const float* Nf = NB[nc];
    for (int ul = lo + tid; ul < hi; ul += nt) {
        int u = r0 + ul;
        int n = s_nrot[ul];
        if (n == 1) {
            b.marg[u * 8] = 1.f;
            for (int k = 1; k < 8; ++k) b.marg[u * 8 + k] = 0.f;
            continue;
        }
        float sum = 0.f;
        for (int k = 0; k < n; ++k) sum += Nf[(ul - nb_lo) * 8 + k];
        float inv = 1.f / sum;
        for (int k = 0; k < 8; ++k) b.marg[u * 8 + k] = k < n ? Nf[(ul - nb_lo) * 8 + k] * inv : 0.f;
    }
    if (b.reuse) {  // leave the final state for the next evaluation's solve
        int* pr = b.prev_row_ptr + size_t(par) * (b.n_res + 1);
        int* pc = b.prev_col + size_t(par) * b.ent_cap;
        float* pm = b.prev_msg + size_t(par) * b.ent_cap * 8;
        const float4* fin = reinterpret_cast<const float4*>(EM[ec]);
        for (int e = eo0 + tid; e < eo1; e += nt) {
            pc[e] = b.col[e];
            reinterpret_cast<float4*>(pm)[2 * e] = fin[2 * e];
            reinterpret_cast<float4*>(pm)[2 * e + 1] = fin[2 * e + 1];
        }
        for (int u = r0 + lo + tid; u <= r0 + hi; u += nt) pr[u] = min(b.row_ptr[u], e1);
        if (tid == 0 && crank == 0) b.prev_valid[par * b.n_sys + s] = 1;
    }
    cluster.sync();  // every node marginal of the system is written
    // Edge marginals of own entries and, when asked, the Bethe free energy
    // (src/rotamer.cpp:292-302, 451-471).  Each entry's 6x6 block is formed in
    // registers from one load of P and the two nodes' cavity beliefs, stored
    // once, and its energy term taken from the same registers: no store is
    // re-read and no load waits behind a store.
    const float* Ef = EM[ec];
    double en = 0.0;
    // Algorithmic bytes of the solve, counted per undirected edge (u < v) of
    // rotamer counts (nu, nv), with ru(n) = n rounded up to 4 floats: every
    // sweep reads and writes both messages and both node beliefs,
    // 4 (2 (ru(nu) + ru(nv)) + 2 ru(nu) + 2 ru(nv)) bytes, and the edge
    // matrix is read once per solve, 4 nu ru(nv) bytes.
    unsigned long long ab_sweep = 0, ab_once = 0;
    for (int e = eo0 + tid; e < eo1; e += nt) {
        const int u = b.erow[e], v = b.col[e];
        const int nu = b.nrot[u], nv = b.nrot[v];
        if (u < v) {
            const unsigned ru = (nu + 3) & ~3, rv = (nv + 3) & ~3;
            ab_sweep += 4ull * (2 * (ru + rv) + 2 * ru + 2 * rv);
            ab_once += 4ull * nu * rv;
        }
        const float4* mu4 = reinterpret_cast<const float4*>(Ef + size_t(e) * 8);
        const float4* mv4 = reinterpret_cast<const float4*>(Ef + size_t(b.rev[e]) * 8);
        const float4* gu4 = reinterpret_cast<const float4*>(b.marg + size_t(u) * 8);
        const float4* gv4 = reinterpret_cast<const float4*>(b.marg + size_t(v) * 8);
        const float4 mu0 = mu4[0], mu1 = mu4[1], mv0 = mv4[0], mv1 = mv4[1];
        const float4 gu0 = gu4[0], gu1 = gu4[1], gv0 = gv4[0], gv1 = gv4[1];
        const float mu[6] = {mu0.x, mu0.y, mu0.z, mu0.w, mu1.x, mu1.y};
        const float mv[6] = {mv0.x, mv0.y, mv0.z, mv0.w, mv1.x, mv1.y};
        const float gu[6] = {gu0.x, gu0.y, gu0.z, gu0.w, gu1.x, gu1.y};
        const float gv[6] = {gv0.x, gv0.y, gv0.z, gv0.w, gv1.x, gv1.y};
        float bu[6], bv[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            bu[i] = i < nu ? gu[i] / (1e-10f + mu[i]) : 0.f;
            bv[i] = i < nv ? gv[i] / (1e-10f + mv[i]) : 0.f;
        }
        // two passes over P's rows (loads only, no store in between): the
        // normalisation, then the normalised block with its energy term
        const float2* P2 = reinterpret_cast<const float2*>(b.P + size_t(e) * 36);
        float sum = 0.f;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            const float2 a0 = P2[3 * i], a1 = P2[3 * i + 1], a2 = P2[3 * i + 2];
            sum += bu[i] * (((a0.x * bv[0] + a0.y * bv[1]) + (a1.x * bv[2] + a1.y * bv[3])) + (a2.x * bv[4] + a2.y * bv[5]));
        }
        const float inv = 1.f / sum;
        float2* mg2 = reinterpret_cast<float2*>(b.emarg + size_t(e) * 36);
        float f = 0.f;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            const float2 a0 = P2[3 * i], a1 = P2[3 * i + 1], a2 = P2[3 * i + 2];
            const float p[6] = {a0.x, a0.y, a1.x, a1.y, a2.x, a2.y};
            float y[6];
#pragma unroll
            for (int j = 0; j < 6; ++j) y[j] = p[j] * bu[i] * bv[j] * inv;
            mg2[3 * i] = make_float2(y[0], y[1]);
            mg2[3 * i + 1] = make_float2(y[2], y[3]);
            mg2[3 * i + 2] = make_float2(y[4], y[5]);
            if (want_energy && u < v && i < nu) {
#pragma unroll
                for (int j = 0; j < 6; ++j)
                    if (j < nv) f += y[j] * logf((1e-10f + y[j]) / (1e-10f + p[j] * gu[i] * gv[j]));
            }
        }
        en += double(f);
    }
    {
        unsigned long long ab = (unsigned long long)(1 + iter) * ab_sweep + ab_once;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ab += __shfl_xor_sync(0xffffffffu, ab, o);
        if (lane == 0 && ab) atomicAdd(&b.alg_bytes[s], ab);
    }
    if (!want_energy) return;  // no shared-memory traffic between blocks after the last barrier
    for (int ul = lo + tid; ul < hi; ul += nt) {
        int u = r0 + ul;
        int n = s_nrot[ul];
        float f = b.eoff[u];
        for (int k = 0; k < n; ++k) {
            float bk = b.marg[u * 8 + k];
            f += bk * logf((1e-10f + bk) / (1e-10f + b.prob[u * 8 + k]));
        }
        en += double(f);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) en += __shfl_xor_sync(0xffffffffu, en, o);
    if (lane == 0) dred[warp] = en;
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        for (int w = 0; w < nw; ++w) t += dred[w];
        *cluster.map_shared_rank(&s_en[crank], 0) = t;
    }
    cluster.sync();
    if (tid == 0 && crank == 0) {
        double t = b.e11[s];
        for (int c = 0; c < BP_CLUSTER; ++c) t += s_en[c];
        energy_out[s] = t;
    }
}

// the solve's launch variants: blocks per system, lanes per node, threads
// per block (clusters of 4, 8 and 16 use smaller blocks so that several
// systems' blocks share an SM)
struct BpVariant {
    const void* fn;
    int cluster, lanes, threads;
};
#define UG_BPV(C, L, T) {reinterpret_cast<const void*>(bp_solve_kernel<C, L, T>), C, L, T}
static const BpVariant* bp_variants() {
    static const BpVariant v[] = {
        UG_BPV(2, 8, 1024), UG_BPV(2, 4, 1024), UG_BPV(2, 16, 1024), UG_BPV(1, 8, 1024), UG_BPV(4, 8, 512),
        UG_BPV(4, 4, 512),  UG_BPV(8, 4, 256),  UG_BPV(8, 8, 256),   UG_BPV(16, 4, 128),
    };
    return v;
}
#undef UG_BPV
int bp_variant_count() { return 9; }
void bp_variant_desc(int i, int* cluster, int* lanes, int* threads) {
    const BpVariant& v = bp_variants()[i];
    *cluster = v.cluster;
    *lanes = v.lanes;
    *threads = v.threads;
}

// Per-node decomposition of the solved free energy for the driver's logs
// (residue_free_energies, residue_entropy<0/1>, rotamer_1body_energy,
// src/rotamer.cpp:292-320, 451-500, 929-1023): every node's own term plus
// half of each of its edges' terms, the 1-1 edges included in the free and
// average energies; and per input, the belief-weighted one-body energies.
__global__ void bp_node_log_kernel(DBP b, const float* p0, const float* p1, const float* p2, const float* p3, int n_in,
                                   int w0, int w1, int w2, int w3) {
    grid_dep_entry();
    for (int u = grid_stride_start(); u < b.n_res; u += grid_stride()) {
        int n = b.nrot[u];
        const float* m = b.marg + u * 8;
        const float* pr = b.prob + u * 8;
        float fe = b.eoff[u], pot = b.eoff[u], ent = 0.f;
        for (int k = 0; k < n; ++k) {
            fe += m[k] * logf((1e-10f + m[k]) / (1e-10f + pr[k]));
            pot -= m[k] * logf(1e-10f + pr[k]);
            ent += m[k] * logf(1e-10f + m[k]);
        }
        if (n > 1) {
            int eb = b.row_ptr[u], ee = min(b.row_ptr[u + 1], b.ent_cap);
            for (int e = eb; e < ee; ++e) {
                int v = b.col[e], nv = b.nrot[v];
                const float* p = b.emarg + size_t(e) * 36;
                const float* P = b.P + size_t(e) * 36;
                const float* mv = b.marg + v * 8;
                float f = 0.f, a = 0.f, h = 0.f;
                for (int i = 0; i < n; ++i)
                    for (int j = 0; j < nv; ++j) {
                        float x = p[i * 6 + j], q = P[i * 6 + j], bb = m[i] * mv[j];
                        f += x * logf((1e-10f + x) / (1e-10f + q * bb));
                        a -= x * logf(1e-10f + q);
                        h += x * logf((1e-10f + x) / (1e-10f + bb));
                    }
                fe += 0.5f * f;
                pot += 0.5f * a;
                ent += 0.5f * h;
            }
        }
        b.log_fe[u] = fe + b.log_e11[u];
        b.log_pot[u] = pot + b.log_e11[u];
        b.log_ent[u] = ent;
    }
    const float* pin[4] = {p0, p1, p2, p3};
    const int w[4] = {w0, w1, w2, w3};
    for (int i = grid_stride_start(); i < b.n_bead; i += grid_stride()) {
        int r = b.bead_res[i], l = b.bead_loc[i];
        float m = b.marg[r * 8 + b.bead_rot[i]];
        for (int k = 0; k < n_in; ++k) atomicAdd(&b.log_1b[size_t(k) * b.n_res + r], m * pin[k][size_t(l) * w[k]]);
    }
}

// bead-edge sensitivities from the marginals, their scatter into the bead
// sensitivities, and 1-body sensitivities (src/rotamer.cpp:1057-1086)
__global__ void bp_sens_kernel(DBP b, DGraph g, float* s0, float* s1, float* s2, float* s3, int n_in, int w0,
                               int w1, int w2, int w3) {
    grid_dep_entry();
    const int ne = *g.n_edge;
    const int dw = g.d1 + g.d2;
    const bool runs = g.d1 <= SCATTER_MAXD;
    const int stride = grid_stride(), first = grid_stride_start() - (threadIdx.x & 31);
    for (int e0 = first; e0 < ne; e0 += stride) {  // warp-uniform trips (run sums)
        const int e = e0 + (threadIdx.x & 31);
        float s = 0.f;
        int key = -1;
        float v1[SCATTER_MAXD];
#pragma unroll
        for (int d = 0; d < SCATTER_MAXD; ++d) v1[d] = 0.f;
        if (e < ne) {
            // the edge's weight, located by the structure stage (bp_edge_energy_kernel)
            const int w = g.eaux[e];
            s = w >= 0 ? b.emarg[w] : w == BP_W_ONE ? 1.f : w == BP_W_NONE ? 0.f : b.marg[BP_W_NODE - w];
            g.esens[e] = s;
        }
        // the graph's adjoint (edge_scatter_kernel) for this edge, here rather
        // than in a kernel of its own
        if (s != 0.f) {
            int2 ij = g.edges[e];
            const float* da = g.deriv + size_t(e) * dw;
            key = g.loc1[ij.x];
            float* p2 = g.sens2 + size_t(g.loc2[ij.y]) * g.w2;
            for (int d = 0; d < g.d2; ++d) atomicAdd(p2 + d, s * da[g.d1 + d]);
            if (runs) {
#pragma unroll
                for (int d = 0; d < SCATTER_MAXD; ++d) v1[d] = d < g.d1 ? s * da[d] : 0.f;
            } else {
                float* p1 = g.sens1 + size_t(key) * g.w1;
                for (int d = 0; d < g.d1; ++d) atomicAdd(p1 + d, s * da[d]);
            }
        }
        if (runs) warp_run_add(g.sens1, g.w1, key, v1, g.d1);
    }
    for (int i = grid_stride_start(); i < b.n_bead; i += grid_stride()) {
        float m = b.marg[b.bead_res[i] * 8 + b.bead_rot[i]];
        int l = b.bead_loc[i];
        atomicAdd(s0 + size_t(l) * w0, m);
        if (n_in > 1) atomicAdd(s1 + size_t(l) * w1, m);
        if (n_in > 2) atomicAdd(s2 + size_t(l) * w2, m);
        if (n_in > 3) atomicAdd(s3 + size_t(l) * w3, m);
    }
}

// The structure of the solve from the bead pair list alone: residue-pair
// entries (CSR rows, reverse entries, descriptors), folded 1-rotamer partner
// energies, the summed pair energies and their probability matrices.  It needs no one-body energy, so the
// engine runs it as soon as the bead positions are known, while the one-body
// inputs are still being computed.  Order: launch_bp_reset, the pair search,
// launch_rotamer_edges (values and marks), launch_bp_structure.
void launch_bp_reset(DBP& b, cudaStream_t st) {
    // n_ent is rewritten only by the entry scan of launch_bp_structure, after
    // this kernel completes
    ug::launch(bp_reset_kernel, EDGE_BLOCKS, 256, 0, st, b);
    if (b.log_fe) cudaMemsetAsync(b.log_e11, 0, sizeof(float) * size_t(b.n_res), st);
}
void launch_rotamer_edges(DBP& b, const DGraph& g, cudaStream_t st) {
    ug::launch(rotamer_edge_kernel, EDGE_BLOCKS, 256, 0, st, g, b);
}
void launch_bp_structure(DBP& b, const DGraph& g, cudaStream_t st) {
    int blocks = EDGE_BLOCKS;
    int rb = min(EDGE_BLOCKS, (b.n_res * 32 + 255) / 256);
    launch_scan(b.row_count, b.row_ptr, b.n_res, b.n_ent, st, nullptr, b.ent_cap, b.status, ST_RES_EDGE_OVERFLOW);
    ug::launch(bp_rows_kernel, rb, 256, 0, st, b);
    ug::launch(bp_edge_energy_kernel, blocks, 256, 0, st, b, g);
    ug::launch(bp_pair_prob_kernel, blocks, 256, 0, st, b);
}

// The rest, after launch_bp_structure: one-body energies, node
// probabilities, warm start, the solve, the logging decomposition and the
// sensitivities, whose bead-edge part is scattered into the bead
// sensitivities here (the rotamer node needs no backward of its own).
void launch_bp(DBP& b, const DGraph& g, const float* const* in, float* const* in_sens, const int* w, int n_in,
               int prev_n_ent, int* scan_total, int want_energy, double* energy_out, const WarmDev* warm,
               const float* pos, const int* atom_off, cudaStream_t st) {
    int blocks = EDGE_BLOCKS;
    (void)prev_n_ent;
    if (b.log_fe) cudaMemsetAsync(b.log_1b, 0, sizeof(float) * size_t(b.n_res) * size_t(n_in), st);
    if (b.res_bead_off) {
        ug::launch(bp_bead_prob_kernel, blocks, 256, 0, st, b, in[0], in[1], in[2], in[3], n_in, w[0], w[1], w[2], w[3]);
    } else {
        ug::launch(bp_bead_energy_kernel, blocks, 256, 0, st, b, in[0], in[1], in[2], in[3], n_in, w[0], w[1], w[2],
                   w[3]);
        ug::launch(bp_node_prob_kernel, blocks, 256, 0, st, b);
    }
    if (warm) launch_warm_start(*warm, pos, atom_off, b.res_off, b.prob, b.nrot, b.n_sys, b.n_res, st);
    const BpVariant& v = bp_variants()[b.variant];
    // Compact layout: room for three times a block's share of nodes and ten
    // entries per residue of its share (equilibrated proteins average six),
    // used when it is no larger than the full layout or when the SMs still
    // hold every block of the launch at once with it.
    size_t smem = bp_solve_smem_bytes(b.max_res_sys);
    {
        static int n_sm = 0, per_sm = 0, per_block = 0, reserved = 0;
        if (!n_sm) {
            int dev = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
            cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
            cudaDeviceGetAttribute(&per_block, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
            cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
            n_sm = std::max(1, n_sm);
        }
        const int N = b.max_res_sys, C = v.cluster;
        int nb_cap = std::min(N, (3 * N + C - 1) / C);
        int msg_cap = (10 * N + C - 1) / C;
        // UPSIDE_GB300_BP_MSG_SLOTS=n caps the message slots (at least 16), so
        // that clusters overflow them and take the global-memory fallback
        static const int slots_cap = [] {
            const char* e = std::getenv("UPSIDE_GB300_BP_MSG_SLOTS");
            return e ? std::max(16, std::atoi(e)) : 0;
        }();
        if (slots_cap) msg_cap = std::min(msg_cap, slots_cap);
        msg_cap = (msg_cap + 3) & ~3;  // keeps the arrays after the destination table 16-byte aligned
        // counts, own beliefs (2 x 8 floats), own messages (2 x 8 floats) and
        // destination table, then own prob rows and first entries, own
        // entries' row and column nodes
        size_t compact = 4 * size_t((N + 3) & ~3) + 64 * size_t(nb_cap) + 68 * size_t(msg_cap) +
                         36 * size_t(nb_cap) + 4 + 8 * size_t(msg_cap);
        int need = (b.n_sys * C + n_sm - 1) / n_sm;  // blocks per SM for a single wave
        cudaFuncAttributes fa;
        size_t stat = cudaFuncGetAttributes(&fa, v.fn) == cudaSuccess ? fa.sharedSizeBytes : size_t(2048);
        long long room = std::min<long long>(per_block, per_sm / std::max(1, need) - reserved) - (long long)stat;
        b.dsm_cap = b.nb_cap = 0;
        if ((compact <= smem || (long long)compact <= room) && msg_cap >= 16 && msg_cap < (1 << 20)) {
            b.dsm_cap = msg_cap;
            b.nb_cap = nb_cap;
            smem = compact;
        }
    }
    if (smem > 48 * 1024) cudaFuncSetAttribute(v.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    // clusters above the portable 8 blocks have to be allowed per kernel
    if (v.cluster > 8) cudaFuncSetAttribute(v.fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    // external records: under stream capture they become event-record nodes
    // that every replay of the graph re-records (a plain record would only
    // order the capture)
    bool timed = b.kt_ev && *b.kt_used + 2 <= b.kt_cap;
    if (timed) cudaEventRecordWithFlags(b.kt_ev[(*b.kt_used)++], st, cudaEventRecordExternal);
    {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(unsigned(b.n_sys) * unsigned(v.cluster));
        cfg.blockDim = dim3(unsigned(v.threads));
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st;
        cudaLaunchAttribute at[2];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = unsigned(v.cluster);
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[1].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = pdl_enabled() ? 2 : 1;
        void* args[] = {&b, &want_energy, &energy_out};
        cudaLaunchKernelExC(&cfg, v.fn, args);
    }
    if (timed) cudaEventRecordWithFlags(b.kt_ev[(*b.kt_used)++], st, cudaEventRecordExternal);
    if (b.log_fe)
        ug::launch(bp_node_log_kernel, blocks, 256, 0, st, b, in[0], in[1], in[2], in[3], n_in, w[0], w[1], w[2], w[3]);
    ug::launch(bp_sens_kernel, blocks, 256, 0, st, b, g, in_sens[0], in_sens[1], in_sens[2], in_sens[3], n_in, w[0],
               w[1], w[2], w[3]);
    (void)scan_total;
}

}  // namespace ug
