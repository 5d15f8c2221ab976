// Surface node and the membrane terms that read it; included by engine.cu
// inside its file-local namespace (it uses the engine's host helpers).
//
// Surface (src/surface.cpp:54-696): the TM residues are those whose N, CA, C
// and CB lie inside the slab tm_min < z < tm_max.  For each of n_rotation
// turns about z (angle a * pi/2 / n_rotation about the TM CBs' xy centre) the
// atoms and their auxiliary points are put on a voxel grid, the surface
// voxels found (method 0: the outermost occupied voxel of each x- and y-row;
// method 1: occupied voxels next to lipid voxels, which a layer-wise flood
// fill grows from the grid border), and within them a finer grid picks the
// outermost CB of each fine row; every picked CB gets a share of a lateral
// force proportional to the surface area.  Output per residue: the fraction
// of turns since the residue was first picked, and the mean picked force
// turned back (x, y).  No derivative flows through the node.
//
// GPU layout.  surface_prep_kernel (a block per system) lists the TM residues
// in order, sums their CB centre in order, and turns every atom through all
// turns in sequence, storing the coordinates each turn sees (the reference
// turns its arrays forth and back, so turn a starts from the coordinates the
// earlier turns' round trips left).  surface_turn_kernel (a block per system
// and turn, all turns at once) builds that turn's grid in shared memory as
// bitmasks over x (one 32-bit word per 32 voxels of a row): occupied voxels,
// lipid voxels and the y-extreme labels; the flood fill runs a warp per
// chain of layers, each pass growing the lipid set by the 3 x 3 neighbourhood
// of the layer's lipid sources and then along rows, until a pass changes
// nothing (the closure is independent of the order of visits).  The fine
// extremes and the picked CBs come from shared-memory atomics: the reference
// picks, per fine row, the last CB in residue order whose fine coordinate
// equals the row's final extreme, which is the largest residue index among
// those CBs.  surface_finish_kernel (a block per system) accumulates the
// turns in order.  Every float step that decides a voxel is rounded
// separately in the reference's order (no contraction), so the decisions are
// those of the CPU restatement at the same coordinates.
//
// State kept between evaluations as the reference keeps it: the TM list
// beyond the current TM count keeps earlier entries, and the final division
// by the turn count runs once per entry of the whole list (a residue listed
// twice is divided twice); residues outside the slab keep their last force.

enum : int { ST_SURFACE_GRID = 8 };  // a turn's grid exceeded the kernel's voxel capacity

struct SurfDev {
    int method, n_rot, n_aux, ngz, snx, sny, snz, cap;  // cap: voxels along x and y the large grid holds
    float tm_min, tm_max, radius, gx, gy, r_gz, area_xz, area_yz, r_nrot;
    const float* aux;           // n_aux x 2 (in units of the radius)
    const float* trig;          // n_rot x 4: cos a, sin a, cos -a, sin -a
    const int* used;            // per system its included residues (system-local)
    const int* used_off;        // n_sys + 1
    const int* res_off;         // n_sys + 1: output rows per system
    const int* cat_off;         // n_sys + 1: rows of the concatenated positions
    const int* index_cb;        // per output row: system-local row of its CB in the positions
    int* tm_list;               // per system n_used (state)
    float* sfx;                 // per output row (state)
    float* sfy;
    int* n_tm;                  // per system
    float* center;              // per system (x, y)
    float* xy;                  // per system n_rot x 4 n_used x 2: turned x, y of each atom per turn
    float* zc;                  // per system 4 n_used: z of each atom
    int* cnt;                   // per system n_rot x n_used: picks of each TM residue per turn
    float* tf;                  // per system n_rot x n_used x 2: its force turned back
    int* tcount;                // per output row
    int* dcount;                // per output row
};

__device__ __forceinline__ float surf_rot_x(float rx, float c, float s, float dx, float dy) {
    return __fsub_rn(__fadd_rn(rx, __fmul_rn(c, dx)), __fmul_rn(s, dy));
}
__device__ __forceinline__ float surf_rot_y(float ry, float c, float s, float dx, float dy) {
    return __fadd_rn(__fadd_rn(ry, __fmul_rn(s, dx)), __fmul_rn(c, dy));
}

// TM residues in order, their CB centre, and every atom's coordinates as
// each turn sees them.  Atom k of a system: k < 3 n_tm the backbone atom k
// (residue k / 3), else the CB of TM residue k - 3 n_tm.  Only the first
// n_tm backbone entries turn (the reference passes the TM count as the size
// of its backbone arrays, src/surface.cpp:240, 664).
__global__ void __launch_bounds__(256) surface_prep_kernel(SurfDev D, int pw, const float* __restrict__ pos) {
    grid_dep_entry();
    const int s = blockIdx.x;
    const int u0 = D.used_off[s], nu = D.used_off[s + 1] - u0;
    const int r0 = D.res_off[s], c0 = D.cat_off[s];
    int* tm = D.tm_list + u0;
    __shared__ int s_warp[8];
    __shared__ int s_base;
    if (threadIdx.x == 0) s_base = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int b = 0; b < nu; b += blockDim.x) {
        const int u = b + threadIdx.x;
        bool in = false;
        if (u < nu) {
            const int nr = D.used[u0 + u];
            auto zin = [&](int row) {
                float z = pos[size_t(c0 + row) * pw + 2];
                return z < D.tm_max && z > D.tm_min;
            };
            in = zin(3 * nr) && zin(3 * nr + 1) && zin(3 * nr + 2) && zin(D.index_cb[r0 + nr]);
        }
        const unsigned m = __ballot_sync(0xffffffffu, in);
        if (lane == 0) s_warp[wid] = __popc(m);
        __syncthreads();
        int before = s_base;
        for (int w = 0; w < wid; ++w) before += s_warp[w];
        if (in) tm[before + __popc(m & ((1u << lane) - 1u))] = D.used[u0 + u];
        __syncthreads();
        if (threadIdx.x == 0)
            for (int w = 0; w < int(blockDim.x >> 5); ++w) s_base += s_warp[w];
        __syncthreads();
    }
    const int ntm = s_base;
    float* zc = D.zc + 4 * size_t(u0);
    float* xy = D.xy + size_t(D.n_rot) * 8 * size_t(u0);
    const int na = 4 * ntm;
    // coordinates of every atom (z is never turned)
    for (int k = threadIdx.x; k < na; k += blockDim.x) {
        const int row = k < 3 * ntm ? 3 * tm[k / 3] + k % 3 : D.index_cb[r0 + tm[k - 3 * ntm]];
        const float* p = pos + size_t(c0 + row) * pw;
        zc[k] = p[2];
        xy[2 * k] = p[0];
        xy[2 * k + 1] = p[1];
    }
    __syncthreads();
    __shared__ float s_c[2];
    if (threadIdx.x == 0) {
        float cx = 0.f, cy = 0.f;
        for (int i = 0; i < ntm; ++i) {
            cx = __fadd_rn(cx, xy[2 * (3 * ntm + i)]);
            cy = __fadd_rn(cy, xy[2 * (3 * ntm + i) + 1]);
        }
        s_c[0] = __fdiv_rn(cx, float(ntm));
        s_c[1] = __fdiv_rn(cy, float(ntm));
        D.n_tm[s] = ntm;
        D.center[2 * s] = s_c[0];
        D.center[2 * s + 1] = s_c[1];
    }
    __syncthreads();
    const float cx = s_c[0], cy = s_c[1];
    for (int k = threadIdx.x; k < na; k += blockDim.x) {
        float x = xy[2 * k], y = xy[2 * k + 1];
        const bool turns = k >= 3 * ntm || k < ntm;
        for (int a = 0; a < D.n_rot; ++a) {
            const float4 t = reinterpret_cast<const float4*>(D.trig)[a];
            float dx = __fsub_rn(x, cx), dy = __fsub_rn(y, cy);
            if (turns && !(dx == 0.f && dy == 0.f)) {
                x = surf_rot_x(cx, t.x, t.y, dx, dy);
                y = surf_rot_y(cy, t.x, t.y, dx, dy);
            }
            // turn 0's slot held the start coordinates, read above by this
            // thread alone
            float* o = xy + (size_t(a) * na + k) * 2;
            o[0] = x;
            o[1] = y;
            dx = __fsub_rn(x, cx);
            dy = __fsub_rn(y, cy);
            if (turns && !(dx == 0.f && dy == 0.f)) {
                x = surf_rot_x(cx, t.z, t.w, dx, dy);
                y = surf_rot_y(cy, t.z, t.w, dx, dy);
            }
        }
    }
}

// the voxel of a point: floor((p - side) * scale) per axis
__device__ __forceinline__ void surf_cell(float x, float y, float z, const float* side, const float* sc, int v[3]) {
    v[0] = int(floorf(__fmul_rn(__fsub_rn(x, side[0]), sc[0])));
    v[1] = int(floorf(__fmul_rn(__fsub_rn(y, side[1]), sc[1])));
    v[2] = int(floorf(__fmul_rn(__fsub_rn(z, side[2]), sc[2])));
}
// valid bits of word w of a row of n voxels
__device__ __forceinline__ unsigned surf_wmask(int w, int n) {
    int b = n - 32 * w;
    return b >= 32 ? 0xffffffffu : (b <= 0 ? 0u : ((1u << b) - 1u));
}
// interior bits (voxels 1 .. n-2) of word w
__device__ __forceinline__ unsigned surf_inner(int w, int n) {
    unsigned m = surf_wmask(w, n - 1);
    if (w == 0) m &= ~1u;
    return m;
}

// Lipid closure of layer k (src/surface.cpp:380-451): empty interior voxels
// with a lipid source among their 3 x 3 neighbours in the layer become lipid
// until none is left; a source is a lipid voxel of the layer that, for the
// tail layers (kr >= 0), is also lipid in layer kr.  One warp; rows are
// updated in place (sets only grow, so any interleaving reaches the same
// closure, and a pass in which no lane changes a row proves it reached).
template <int SURF_WMAX>  // words per row the fill keeps in registers (W <= SURF_WMAX)
__device__ void surf_fill(volatile unsigned* L, const unsigned* A, int k, int kr, int ngx, int ngy, int W, int lane) {
    const int max_pass = ngx * ngy + 2;
    for (int pass = 0; pass < max_pass; ++pass) {
        bool changed = false;
        for (int j = 1 + lane; j < ngy - 1; j += 32) {
            volatile unsigned* row = L + size_t(k * ngy + j) * W;
            unsigned src[3][SURF_WMAX];
            for (int dj = 0; dj < 3; ++dj) {
                const volatile unsigned* rr = L + size_t(k * ngy + j - 1 + dj) * W;
                const volatile unsigned* rf = kr >= 0 ? L + size_t(kr * ngy + j - 1 + dj) * W : nullptr;
#pragma unroll
                for (int w = 0; w < SURF_WMAX; ++w)
                    if (w < W) src[dj][w] = rf ? (rr[w] & rf[w]) : rr[w];
            }
            unsigned cur[SURF_WMAX], E[SURF_WMAX], ref_row[SURF_WMAX];
            const unsigned* arow = A + size_t(k * ngy + j) * W;
            const volatile unsigned* rref = kr >= 0 ? L + size_t(kr * ngy + j) * W : nullptr;
#pragma unroll
            for (int w = 0; w < SURF_WMAX; ++w) {
                if (w >= W) continue;
                cur[w] = row[w];
                E[w] = ~arow[w] & ~cur[w] & surf_inner(w, ngx);
                ref_row[w] = rref ? rref[w] : 0xffffffffu;
                unsigned d = 0;
                for (int dj = 0; dj < 3; ++dj) {
                    unsigned x = src[dj][w];
                    d |= x | (x << 1) | (x >> 1);
                    if (w > 0) d |= src[dj][w - 1] >> 31;
                    if (w + 1 < W) d |= src[dj][w + 1] << 31;
                }
                cur[w] |= E[w] & d;
            }
            // along the row: new lipid voxels that are sources spread further
            for (int it = 0; it < ngx; ++it) {
                bool grew = false;
                unsigned nxt[SURF_WMAX];
#pragma unroll
                for (int w = 0; w < SURF_WMAX; ++w) {
                    if (w >= W) continue;
                    unsigned x = cur[w] & ref_row[w];
                    unsigned d = x | (x << 1) | (x >> 1);
                    if (w > 0) d |= (cur[w - 1] & ref_row[w - 1]) >> 31;
                    if (w + 1 < W) d |= (cur[w + 1] & ref_row[w + 1]) << 31;
                    nxt[w] = cur[w] | (E[w] & d);
                    grew |= nxt[w] != cur[w];
                }
                if (!grew) break;
#pragma unroll
                for (int w = 0; w < SURF_WMAX; ++w)
                    if (w < W) cur[w] = nxt[w];
            }
#pragma unroll
            for (int w = 0; w < SURF_WMAX; ++w) {
                if (w >= W) continue;
                if (cur[w] != row[w]) {
                    row[w] = cur[w];
                    changed = true;
                }
            }
        }
        __syncwarp();
        if (!__any_sync(0xffffffffu, changed)) break;
    }
}

// block-wide reductions over 256 threads (8 warps)
__device__ __forceinline__ float surf_bmin(float v, float* sh) {
    for (int o = 16; o; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    float r = sh[0];
    for (int w = 1; w < 8; ++w) r = fminf(r, sh[w]);
    return r;
}
__device__ __forceinline__ int surf_bsum(int v, int* sh) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    int r = 0;
    for (int w = 0; w < 8; ++w) r += sh[w];
    return r;
}

// One turn of one system (src/surface.cpp:234-673), on a grid of at most
// cap x cap voxels in x and y (cap <= 32 WMAX).  Two tiers: the small grid
// runs every turn and leaves the turns whose grid is larger to the large one
// (big[] flags, per system and turn); the large tier skips all others.
// Dynamic shared memory: three masks of ngz x cap rows x cap/32 words
// (occupied; lipid or y-minimum labels; y-maximum labels) and the fine
// extremes and picks.
template <int WMAX>
__global__ void __launch_bounds__(256, WMAX <= 2 ? 4 : 1) surface_turn_kernel(SurfDev D, int cap, int tier, int* big, int* status) {
    grid_dep_entry();
    extern __shared__ unsigned smem_u[];
    const int a = blockIdx.x, s = blockIdx.y, tid = threadIdx.x, bd = blockDim.x;
    if (tier == 1 && !big[s * D.n_rot + a]) return;
    const int u0 = D.used_off[s], nu = D.used_off[s + 1] - u0;
    const int ntm = D.n_tm[s];
    int* cnt = D.cnt + size_t(D.n_rot) * u0 + size_t(a) * nu;
    float* tf = D.tf + (size_t(D.n_rot) * u0 + size_t(a) * nu) * 2;
    for (int i = tid; i < ntm; i += bd) cnt[i] = 0;
    if (ntm == 0) {
        if (tid == 0 && tier == 0) big[s * D.n_rot + a] = 0;
        return;
    }
    const int na = 4 * ntm;
    const float* xy = D.xy + size_t(D.n_rot) * 8 * size_t(u0) + size_t(a) * na * 2;
    const float* zc = D.zc + 4 * size_t(u0);
    __shared__ float s_red[8];
    __shared__ int s_ired[8];
    __shared__ int s_g[6];       // ngx, ngy, W, skip, big, zs
    __shared__ float s_f[13];    // side[3], s1[3], s2[3], forces xmin, xmax, ymin, ymax
    // 1. extent of the turned atoms (src/surface.cpp:242-255)
    float mnx = INFINITY, mxx = -INFINITY, mny = INFINITY, mxy = -INFINITY;
    for (int k = tid; k < na; k += bd) {
        float x = xy[2 * k], y = xy[2 * k + 1];
        mnx = fminf(mnx, x);
        mxx = fmaxf(mxx, x);
        mny = fminf(mny, y);
        mxy = fmaxf(mxy, y);
    }
    mnx = surf_bmin(mnx, s_red);
    mxx = -surf_bmin(-mxx, s_red);
    mny = surf_bmin(mny, s_red);
    mxy = -surf_bmin(-mxy, s_red);
    // 2. the grid (src/surface.cpp:257-270), in the reference's roundings
    if (tid == 0) {
        float minx = __fsub_rn(mnx, D.radius), maxx = __fadd_rn(mxx, D.radius);
        float miny = __fsub_rn(mny, D.radius), maxy = __fadd_rn(mxy, D.radius);
        float lenx = __fsub_rn(maxx, minx), leny = __fsub_rn(maxy, miny);
        double qx = __ddiv_rn(__dadd_rn(double(lenx), 0.1), double(D.gx));
        double qy = __ddiv_rn(__dadd_rn(double(leny), 0.1), double(D.gy));
        bool ok = qx >= 0. && qy >= 0. && qx < double(cap) && qy < double(cap);
        int ngx = ok ? int(qx) + 3 : 3, ngy = ok ? int(qy) + 3 : 3;
        ok = ok && ngx <= cap && ngy <= cap;
        float blx = __fmul_rn(float(ngx), D.gx), bly = __fmul_rn(float(ngy), D.gy);
        s_f[0] = __fsub_rn(minx, __fmul_rn(0.5f, __fsub_rn(blx, lenx)));
        s_f[1] = __fsub_rn(miny, __fmul_rn(0.5f, __fsub_rn(bly, leny)));
        s_f[2] = __fsub_rn(D.tm_min, D.radius);
        s_f[3] = __fdiv_rn(float(ngx), blx);
        s_f[4] = __fdiv_rn(float(ngy), bly);
        s_f[5] = D.r_gz;
        s_f[6] = __fdiv_rn(float(D.snx * ngx), blx);
        s_f[7] = __fdiv_rn(float(D.sny * ngy), bly);
        s_f[8] = __fmul_rn(float(D.snz), D.r_gz);
        s_g[0] = ngx;
        s_g[1] = ngy;
        s_g[2] = (ngx + 31) >> 5;
        s_g[3] = ok ? 0 : 1;
        s_g[4] = ngx * D.snx + ngy * D.sny + D.ngz * D.snz;
        s_g[5] = D.ngz * D.snz;
        // a finite extent beyond the small grid goes to the large tier; beyond
        // the large grid, or not finite, it is an error
        const bool finite = qx >= 0. && qy >= 0. && qx < 1e9 && qy < 1e9;
        if (tier == 0) big[s * D.n_rot + a] = (!ok && finite) ? 1 : 0;
        if (!ok && (tier == 1 || !finite)) atomicOr(status, ST_SURFACE_GRID);
    }
    __syncthreads();
    const int ngx = s_g[0], ngy = s_g[1], W = s_g[2], big_int = s_g[4], zs = s_g[5], ngz = D.ngz;
    if (s_g[3]) {
        for (int i = tid; i < ntm; i += bd) tf[2 * i] = tf[2 * i + 1] = 0.f;
        return;
    }
    const float side[3] = {s_f[0], s_f[1], s_f[2]}, s1[3] = {s_f[3], s_f[4], s_f[5]}, s2[3] = {s_f[6], s_f[7], s_f[8]};
    const int nrow = ngz * ngy, nword = nrow * W;
    const size_t mcap = size_t(ngz) * cap * (cap / 32);
    unsigned* A = smem_u;
    unsigned* M2 = A + mcap;  // method 1: lipid; method 0: y-minimum labels
    unsigned* M3 = M2 + mcap; // method 0: y-maximum labels
    const int nfx = D.sny * ngy * zs, nfy = D.snx * ngx * zs;
    const size_t fcx = size_t(D.sny) * cap * size_t(D.ngz * D.snz), fcy = size_t(D.snx) * cap * size_t(D.ngz * D.snz);
    int* fxmn = reinterpret_cast<int*>(M3 + mcap);
    int* fxmx = fxmn + fcx;
    int* ixmn = fxmx + fcx;
    int* ixmx = ixmn + fcx;
    int* fymn = ixmx + fcx;
    int* fymx = fymn + fcy;
    int* iymn = fymx + fcy;
    int* iymx = iymn + fcy;
    for (int i = tid; i < nword; i += bd) A[i] = M2[i] = M3[i] = 0u;
    for (int i = tid; i < nfx; i += bd) { fxmn[i] = big_int; fxmx[i] = -1; ixmn[i] = ixmx[i] = -1; }
    for (int i = tid; i < nfy; i += bd) { fymn[i] = big_int; fymx[i] = -1; iymn[i] = iymx[i] = -1; }
    __syncthreads();
    // 3. occupied voxels: atoms and their auxiliary points (src/surface.cpp:272-321)
    const int per = 1 + 2 * D.n_aux;
    auto point = [&](int k, int j, float& x, float& y, float& z) {
        x = xy[2 * k];
        y = xy[2 * k + 1];
        z = zc[k];
        if (j > 0) {
            const int q = j <= D.n_aux ? j - 1 : j - 1 - D.n_aux;
            const float o0 = __fmul_rn(D.aux[2 * q], D.radius), o1 = __fmul_rn(D.aux[2 * q + 1], D.radius);
            if (j <= D.n_aux) y = __fadd_rn(y, o0);
            else x = __fadd_rn(x, o0);
            z = __fadd_rn(z, o1);
        }
    };
    for (int p = tid; p < na * per; p += bd) {
        const int k = p / per, j = p - k * per;
        float x, y, z;
        point(k, j, x, y, z);
        int v[3];
        surf_cell(x, y, z, side, s1, v);
        if (v[0] < 0 || v[1] < 0 || v[2] < 0 || v[0] >= ngx || v[1] >= ngy || v[2] >= ngz) {
            atomicOr(status, ST_SURFACE_GRID);
            continue;
        }
        atomicOr(&A[(v[2] * ngy + v[1]) * W + (v[0] >> 5)], 1u << (v[0] & 31));
    }
    __syncthreads();
    // 4. surface voxels (src/surface.cpp:323-468)
    if (D.method == 1) {
        // grid border: lipid (src/surface.cpp:368-378)
        for (int i = tid; i < nword; i += bd) {
            const int r = i / W, w = i - r * W, j = r % ngy;
            unsigned b = (j == 0 || j == ngy - 1) ? surf_wmask(w, ngx) : (surf_wmask(w, ngx) & ~surf_inner(w, ngx));
            M2[i] = b;
            A[i] &= ~b;
        }
        __syncthreads();
        const int lane = tid & 31, wid = tid >> 5;
        if (wid == 0) {
            surf_fill<WMAX>(M2, A, 0, -1, ngx, ngy, W, lane);
            for (int k = 1; k < ngz / 2; ++k) surf_fill<WMAX>(M2, A, k, k - 1, ngx, ngy, W, lane);
        } else if (wid == 1) {
            // the reference's pass over the top layer with the layer above
            // it (read past its grid) cannot add to a layer closed just before
            surf_fill<WMAX>(M2, A, ngz - 1, -1, ngx, ngy, W, lane);
            for (int k = ngz - 2; k >= ngz / 2; --k) surf_fill<WMAX>(M2, A, k, k + 1, ngx, ngy, W, lane);
        }
    } else {
        // per column the first and last occupied voxel along y
        for (int t = tid; t < ngz * W; t += bd) {
            const int k = t / W, w = t - k * W;
            unsigned seen = 0u;
            for (int j = 0; j < ngy; ++j) {
                const int i = (k * ngy + j) * W + w;
                M2[i] = A[i] & ~seen;
                seen |= A[i];
            }
            seen = 0u;
            for (int j = ngy - 1; j >= 0; --j) {
                const int i = (k * ngy + j) * W + w;
                M3[i] = A[i] & ~seen;
                seen |= A[i];
            }
        }
    }
    __syncthreads();
    // labels of an occupied voxel: bit 0 x-min, 1 x-max, 2 y-min, 3 y-max face
    auto labels = [&](const int* v) -> int {
        const int r = v[2] * ngy + v[1];
        const unsigned* row = A + size_t(r) * W;
        if (!((row[v[0] >> 5] >> (v[0] & 31)) & 1u)) return 0;
        auto bit = [&](const unsigned* m, int rr, int i) { return int((m[size_t(rr) * W + (i >> 5)] >> (i & 31)) & 1u); };
        if (D.method == 1) {
            if (v[0] < 1 || v[0] > ngx - 2 || v[1] < 1 || v[1] > ngy - 2) return 0;
            return bit(M2, r, v[0] - 1) | (bit(M2, r, v[0] + 1) << 1) | (bit(M2, r - 1, v[0]) << 2) |
                   (bit(M2, r + 1, v[0]) << 3);
        }
        int lo = -1, hi = -1;
        for (int w = 0; w < W && lo < 0; ++w)
            if (row[w]) lo = 32 * w + __ffs(row[w]) - 1;
        for (int w = W - 1; w >= 0 && hi < 0; --w)
            if (row[w]) hi = 32 * w + 31 - __clz(row[w]);
        return int(v[0] == lo) | (int(v[0] == hi) << 1) | (bit(M2, r, v[0]) << 2) | (bit(M3, r, v[0]) << 3);
    };
    // 5. fine extremes over the surface atoms, their auxiliary points and the
    // CBs' auxiliary points and CBs (src/surface.cpp:471-594): a thread per
    // atom; only atoms in a surface voxel go through their points
    for (int k = tid; k < na; k += bd) {
        float x, y, z;
        point(k, 0, x, y, z);
        int v[3], q[3];
        surf_cell(x, y, z, side, s1, v);
        if (v[0] < 0 || v[1] < 0 || v[2] < 0 || v[0] >= ngx || v[1] >= ngy || v[2] >= ngz) continue;
        const int lab = labels(v);
        if (!lab) continue;
        surf_cell(x, y, z, side, s2, q);
        for (int j = 0; j < per; ++j) {
            int c[3];
            if (j == 0) {
                c[0] = q[0]; c[1] = q[1];
            } else {
                float px, py, pz;
                point(k, j, px, py, pz);
                surf_cell(px, py, pz, side, s2, c);
            }
            if (j <= D.n_aux) {  // the point itself or a y-offset point: x extremes of its fine row
                const int kj = c[1] * zs + q[2];
                if (kj < 0 || kj >= nfx) { atomicOr(status, ST_SURFACE_GRID); continue; }
                if (lab & 1) atomicMin(&fxmn[kj], c[0]);
                if (lab & 2) atomicMax(&fxmx[kj], c[0]);
            }
            if (j == 0 || j > D.n_aux) {  // the point itself or an x-offset point: y extremes
                const int ki = c[0] * zs + q[2];
                if (ki < 0 || ki >= nfy) { atomicOr(status, ST_SURFACE_GRID); continue; }
                if (lab & 4) atomicMin(&fymn[ki], c[1]);
                if (lab & 8) atomicMax(&fymx[ki], c[1]);
            }
        }
    }
    __syncthreads();
    // picks: per fine row the last CB in residue order at the final extreme
    for (int nr = tid; nr < ntm; nr += bd) {
        const int k = 3 * ntm + nr;
        float x, y, z;
        point(k, 0, x, y, z);
        int v[3], q[3];
        surf_cell(x, y, z, side, s1, v);
        if (v[0] < 0 || v[1] < 0 || v[2] < 0 || v[0] >= ngx || v[1] >= ngy || v[2] >= ngz) continue;
        const int lab = labels(v);
        if (!lab) continue;
        surf_cell(x, y, z, side, s2, q);
        const int kj = q[1] * zs + q[2], ki = q[0] * zs + q[2];
        if (kj >= 0 && kj < nfx) {
            if ((lab & 1) && q[0] == fxmn[kj]) atomicMax(&ixmn[kj], nr);
            if ((lab & 2) && q[0] == fxmx[kj]) atomicMax(&ixmx[kj], nr);
        }
        if (ki >= 0 && ki < nfy) {
            if ((lab & 4) && q[1] == fymn[ki]) atomicMax(&iymn[ki], nr);
            if ((lab & 8) && q[1] == fymx[ki]) atomicMax(&iymx[ki], nr);
        }
    }
    __syncthreads();
    // 6. areas and forces per picked CB (src/surface.cpp:596-622)
    int n_xmn = 0, n_xmx = 0, n_ymn = 0, n_ymx = 0, c_xmn = 0, c_xmx = 0, c_ymn = 0, c_ymx = 0;
    for (int i = tid; i < nfx; i += bd) {
        n_xmn += fxmn[i] < big_int;
        n_xmx += fxmx[i] > -1;
        if (ixmn[i] >= 0) { ++c_xmn; atomicOr(&cnt[ixmn[i]], 1); }
        if (ixmx[i] >= 0) { ++c_xmx; atomicAdd(&cnt[ixmx[i]], 4); }
    }
    for (int i = tid; i < nfy; i += bd) {
        n_ymn += fymn[i] < big_int;
        n_ymx += fymx[i] > -1;
        if (iymn[i] >= 0) { ++c_ymn; atomicOr(&cnt[iymn[i]], 2); }
        if (iymx[i] >= 0) { ++c_ymx; atomicAdd(&cnt[iymx[i]], 1 << 16); }
    }
    n_xmn = surf_bsum(n_xmn, s_ired);
    n_xmx = surf_bsum(n_xmx, s_ired);
    n_ymn = surf_bsum(n_ymn, s_ired);
    n_ymx = surf_bsum(n_ymx, s_ired);
    c_xmn = surf_bsum(c_xmn, s_ired);
    c_xmx = surf_bsum(c_xmx, s_ired);
    c_ymn = surf_bsum(c_ymn, s_ired);
    c_ymx = surf_bsum(c_ymx, s_ired);
    if (tid == 0) {
        float a_xmn = __fmul_rn(float(n_xmn), D.area_yz), a_xmx = __fmul_rn(float(n_xmx), D.area_yz);
        float a_ymn = __fmul_rn(float(n_ymn), D.area_xz), a_ymx = __fmul_rn(float(n_ymx), D.area_xz);
        float ax = a_xmn > a_xmx ? a_xmn : a_xmx, ay = a_ymn > a_ymx ? a_ymn : a_ymx;
        // FORCE_UNIT is a double literal in the reference (src/surface.cpp:15)
        float tfx = __double2float_rn(__dmul_rn(double(ax), 2.428602e-5));
        float tfy = __double2float_rn(__dmul_rn(double(ay), 2.428602e-5));
        s_f[9] = __fdiv_rn(tfx, float(c_xmn));
        s_f[10] = __fdiv_rn(tfx, float(c_xmx));
        s_f[11] = __fdiv_rn(tfy, float(c_ymn));
        s_f[12] = __fdiv_rn(tfy, float(c_ymx));
    }
    __syncthreads();
    // 7. each TM residue's force of this turn, turned back (src/surface.cpp:624-672)
    const float4 t = reinterpret_cast<const float4*>(D.trig)[a];
    for (int nr = tid; nr < ntm; nr += bd) {
        const int c = cnt[nr];
        float fx = (c & 1) ? s_f[9] : 0.f, fy = (c & 2) ? s_f[11] : 0.f;
        for (int i = (c >> 2) & 0x3fff; i > 0; --i) fx = __fsub_rn(fx, s_f[10]);
        for (int i = c >> 16; i > 0; --i) fy = __fsub_rn(fy, s_f[12]);
        if (!(fx == 0.f && fy == 0.f)) {
            const float rx = surf_rot_x(0.f, t.z, t.w, fx, fy);
            fy = surf_rot_y(0.f, t.z, t.w, fx, fy);
            fx = rx;
        }
        tf[2 * nr] = fx;
        tf[2 * nr + 1] = fy;
    }
}

// The turns in order (src/surface.cpp:666-690): a residue counts every turn
// from the first that picks it; its force sums the turned-back forces of
// those turns and is divided by that count once per entry of the whole TM
// list; output (fraction of turns, force x, force y) for every residue.
__global__ void __launch_bounds__(256) surface_finish_kernel(SurfDev D, float* out) {
    grid_dep_entry();
    const int s = blockIdx.x, tid = threadIdx.x, bd = blockDim.x;
    const int u0 = D.used_off[s], nu = D.used_off[s + 1] - u0;
    const int r0 = D.res_off[s], nres = D.res_off[s + 1] - r0;
    const int ntm = D.n_tm[s];
    const int* tm = D.tm_list + u0;
    const int* cnt = D.cnt + size_t(D.n_rot) * u0;
    const float* tf = D.tf + size_t(D.n_rot) * u0 * 2;
    for (int r = tid; r < nres; r += bd) D.tcount[r0 + r] = D.dcount[r0 + r] = 0;
    __syncthreads();
    for (int u = tid; u < nu; u += bd) atomicAdd(&D.dcount[r0 + tm[u]], 1);
    for (int ns = tid; ns < ntm; ns += bd) {
        int first = -1;
        float sx = 0.f, sy = 0.f;
        for (int a = 0; a < D.n_rot; ++a) {
            if (first < 0 && cnt[size_t(a) * nu + ns]) first = a;
            if (first >= 0) {
                sx = __fadd_rn(sx, tf[(size_t(a) * nu + ns) * 2]);
                sy = __fadd_rn(sy, tf[(size_t(a) * nu + ns) * 2 + 1]);
            }
        }
        const int nr = tm[ns];
        D.tcount[r0 + nr] = first >= 0 ? D.n_rot - first : 0;
        D.sfx[r0 + nr] = sx;
        D.sfy[r0 + nr] = sy;
    }
    __syncthreads();
    for (int ns = tid; ns < ntm; ns += bd) {
        const int nr = tm[ns], t = D.tcount[r0 + nr];
        if (t <= 0) continue;
        float sx = D.sfx[r0 + nr], sy = D.sfy[r0 + nr];
        for (int i = D.dcount[r0 + nr]; i > 0; --i) {
            sx = __fdiv_rn(sx, float(t));
            sy = __fdiv_rn(sy, float(t));
        }
        D.sfx[r0 + nr] = sx;
        D.sfy[r0 + nr] = sy;
    }
    __syncthreads();
    for (int r = tid; r < nres; r += bd) {
        const int t = D.tcount[r0 + r];
        float* o = out + size_t(r0 + r) * 3;
        o[0] = t > 0 ? __fmul_rn(float(t), D.r_nrot) : 0.f;
        o[1] = D.sfx[r0 + r];
        o[2] = D.sfy[r0 + r];
    }
}

constexpr int SURF_W_SMALL = 2, SURF_W_LARGE = 7;  // words per grid row of the two tiers (64 and 224 voxels)

struct SurfaceNode : GNode {
    SurfDev D{};
    int n_sys = 0;
    int cap_small = 0, cap_large = 0;
    size_t smem_small = 0, smem_large = 0;
    int* big = nullptr;
    size_t n_used_total = 0;
    int *snap_tm = nullptr;
    float* snap_sf = nullptr;
    // argument: the concatenated backbone and CB positions (cat_pos)
    SurfaceNode(Engine& e, const Groups& g, const GNode& pos) {
        width = 3;
        n_sys = int(g.size());
        D.method = int(shared_attr(g, "method_type"));
        if (D.method != 0 && D.method != 1) throw Error("surface method_type must be 0 or 1");
        D.n_rot = int(shared_attr(g, "n_rotation"));
        if (D.n_rot < 1) throw Error("surface needs n_rotation >= 1");
        const float half = float(shared_attr(g, "half_thickness")), zbuf = float(shared_attr(g, "zbuffer"));
        D.radius = float(shared_attr(g, "atom_radius"));
        D.tm_min = -half - zbuf;
        D.tm_max = half + zbuf;
        D.ngz = int(shared_attr(g, "n_gridz"));
        if (D.ngz < 2) throw Error("surface needs n_gridz >= 2");
        D.gx = float(shared_attr(g, "len_gridx"));
        D.gy = float(shared_attr(g, "len_gridy"));
        if (!(D.gx > 0.f) || !(D.gy > 0.f)) throw Error("surface grid lengths must be positive");
        // GRID_Z = (tm_max - tm_min + 2 radius + 0.1) / n_gridz, the 0.1 a
        // double literal (src/surface.cpp:122)
        float ext = D.tm_max - D.tm_min;
        ext = ext + float(2) * D.radius;
        const float gz = float((double(ext) + 0.1) / D.ngz);
        D.r_gz = 1.f / gz;
        D.snx = int(shared_attr(g, "n_smallgridx"));
        D.sny = int(shared_attr(g, "n_smallgridy"));
        D.snz = int(shared_attr(g, "n_smallgridz"));
        if (D.snx < 1 || D.sny < 1 || D.snz < 1) throw Error("surface small grids need at least one cell");
        D.area_xz = D.gx / float(D.snx) * gz / float(D.snz);
        D.area_yz = D.gy / float(D.sny) * gz / float(D.snz);
        D.r_nrot = float(1. / D.n_rot);
        auto aux = shared_f(g, "auxiliary_point");
        auto ad = g.f(0).dims(g.p("auxiliary_point"));
        if (ad.size() != 2 || ad[1] != 2) throw Error("auxiliary_point must be (n_aux, 2)");
        D.n_aux = int(ad[0]);
        D.aux = e.upload(aux.empty() ? std::vector<float>(2, 0.f) : aux);
        // turn angles a * (pi/2 / n_rotation) in float and their cosines and
        // sines from the host's libm, as the reference takes them
        const float step = float(0.5 * double(3.141592653589793f) * double(D.r_nrot));
        std::vector<float> trig;
        for (int a = 0; a < D.n_rot; ++a) {
            const float ang = float(a) * step;
            trig.push_back(std::cos(ang));
            trig.push_back(std::sin(ang));
            trig.push_back(std::cos(-ang));
            trig.push_back(std::sin(-ang));
        }
        D.trig = e.upload(trig);
        // residues, their CB rows and the included list per system
        std::vector<int> res_c, used, used_c, icb;
        for (size_t s = 0; s < g.size(); ++s) {
            auto cb = read_i(g.f(s), g.p("index_cb"));
            const int nres = int(cb.size()), rows = pos.off[s + 1] - pos.off[s];
            for (int r = 0; r < nres; ++r) {
                if (cb[size_t(r)] < 0 || cb[size_t(r)] >= rows || 3 * r + 2 >= rows)
                    throw Error("surface index_cb row " + std::to_string(cb[size_t(r)]) + " or backbone of residue " +
                                std::to_string(r) + " outside the " + std::to_string(rows) + " positions");
                icb.push_back(cb[size_t(r)]);
            }
            res_c.push_back(nres);
            const int excl = int(attr_d(g.f(s), g.path, "exclusion"));
            std::vector<int> u;
            if (excl == 1) u = read_i(g.f(s), g.p("included_list"));
            else
                for (int r = 0; r < nres; ++r) u.push_back(r);
            for (int r : u)
                if (r < 0 || r >= nres) throw Error("surface included_list entry " + std::to_string(r) + " out of range");
            used.insert(used.end(), u.begin(), u.end());
            used_c.push_back(int(u.size()));
        }
        off = offsets(res_c);
        total = off.back();
        auto uoff = offsets(used_c);
        n_used_total = size_t(uoff.back());
        D.used = e.upload(used.empty() ? std::vector<int>(1, 0) : used);
        D.used_off = e.upload(uoff);
        D.res_off = e.upload(off);
        D.cat_off = e.upload(pos.off);
        D.index_cb = e.upload(icb.empty() ? std::vector<int>(1, 0) : icb);
        const size_t nu = std::max<size_t>(1, n_used_total), nr = std::max(1, total);
        D.tm_list = e.alloc<int>(nu);
        D.sfx = e.alloc<float>(nr);
        D.sfy = e.alloc<float>(nr);
        UG_CK(cudaMemsetAsync(D.tm_list, 0, 4 * nu, e.st));
        UG_CK(cudaMemsetAsync(D.sfx, 0, 4 * nr, e.st));
        UG_CK(cudaMemsetAsync(D.sfy, 0, 4 * nr, e.st));
        D.n_tm = e.alloc<int>(size_t(n_sys));
        D.center = e.alloc<float>(2 * size_t(n_sys));
        D.xy = e.alloc<float>(size_t(D.n_rot) * 8 * nu);
        D.zc = e.alloc<float>(4 * nu);
        D.cnt = e.alloc<int>(size_t(D.n_rot) * nu);
        D.tf = e.alloc<float>(size_t(D.n_rot) * 2 * nu);
        D.tcount = e.alloc<int>(nr);
        D.dcount = e.alloc<int>(nr);
        snap_tm = e.alloc<int>(nu);
        snap_sf = e.alloc<float>(2 * nr);
        // per tier the largest square grid (a multiple of 32 voxels, at most
        // 32 words per row of the tier) whose masks and fine rows fit in a
        // block's shared memory
        auto fit = [&](int wmax, int& cap, size_t& bytes) {
            const size_t limit = 200 * 1024;
            for (int c = 32 * wmax; c >= 32; c -= 32) {
                const size_t masks = 3 * size_t(D.ngz) * c * (c / 32) * 4;
                const size_t fine = 4 * 4 * size_t(D.ngz * D.snz) * c * size_t(D.sny + D.snx);
                if (masks + fine <= limit && size_t(D.sny) * c * D.ngz * D.snz < 16384 &&
                    size_t(D.snx) * c * D.ngz * D.snz < 16384) {
                    cap = c;
                    bytes = masks + fine;
                    return;
                }
            }
            throw Error("surface grid parameters leave no room for a voxel grid in shared memory");
        };
        fit(SURF_W_SMALL, cap_small, smem_small);
        fit(SURF_W_LARGE, cap_large, smem_large);
        D.cap = cap_large;
        big = e.alloc<int>(size_t(n_sys) * D.n_rot);
        UG_CK(cudaFuncSetAttribute(surface_turn_kernel<SURF_W_SMALL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   int(smem_small)));
        UG_CK(cudaFuncSetAttribute(surface_turn_kernel<SURF_W_LARGE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   int(smem_large)));
    }
    void forward(Engine& e, bool) override {
        auto& p = e.arg(*this, 0);
        ug::launch(surface_prep_kernel, n_sys, 256, 0, e.st, D, p.width, p.out);
        ug::launch(surface_turn_kernel<SURF_W_SMALL>, dim3(D.n_rot, n_sys), 256, smem_small, e.st, D, cap_small, 0, big,
                   e.d_status);
        ug::launch(surface_turn_kernel<SURF_W_LARGE>, dim3(D.n_rot, n_sys), 256, smem_large, e.st, D, cap_large, 1, big,
                   e.d_status);
        ug::launch(surface_finish_kernel, n_sys, 256, 0, e.st, D, out);
    }
    // the state the next evaluation reads (TM list, forces of every residue)
    void keep_state(Engine& e, bool restore) override {
        const size_t nu = std::max<size_t>(1, n_used_total), nr = std::max(1, total);
        if (restore) {
            UG_CK(cudaMemcpyAsync(D.tm_list, snap_tm, 4 * nu, cudaMemcpyDeviceToDevice, e.st));
            UG_CK(cudaMemcpyAsync(D.sfx, snap_sf, 4 * nr, cudaMemcpyDeviceToDevice, e.st));
            UG_CK(cudaMemcpyAsync(D.sfy, snap_sf + nr, 4 * nr, cudaMemcpyDeviceToDevice, e.st));
        } else {
            UG_CK(cudaMemcpyAsync(snap_tm, D.tm_list, 4 * nu, cudaMemcpyDeviceToDevice, e.st));
            UG_CK(cudaMemcpyAsync(snap_sf, D.sfx, 4 * nr, cudaMemcpyDeviceToDevice, e.st));
            UG_CK(cudaMemcpyAsync(snap_sf + nr, D.sfy, 4 * nr, cudaMemcpyDeviceToDevice, e.st));
        }
    }
};

// ================================================ surface membrane terms ===
// CB term with the surface score (MembraneSurfCBPotential,
// src/membrane_potential.cpp:674-983): as the CB membrane term, but inside the
// slab (and for the first burial bin everywhere) each bin's depth spline is
// weighted by the residue's surface fraction s and the residue type's inner
// spline by 1 - s
__global__ void memb_surf_cb_kernel(int n, MembParams P, float half, int n_rt, int n_bl, const int* __restrict__ cb_row,
                                    const int* __restrict__ env_row, const int* __restrict__ cc_row,
                                    const int* __restrict__ s_row, const int* __restrict__ rtype,
                                    const int* __restrict__ sys, const float* __restrict__ wts,
                                    const float* __restrict__ bl_nodes, const float* __restrict__ coeff,
                                    const float* __restrict__ coeff_in, int cbw, const float* __restrict__ cb,
                                    float* cbs, int ew, const float* __restrict__ env, float* envs, int sw,
                                    const float* __restrict__ surf, const float* __restrict__ cc, double* pot) {
    grid_dep_entry();
    for (int i = grid_stride_start(); i < n; i += grid_stride()) {
        const size_t er = size_t(env_row[i]);
        float bl = 0.f;
        for (int a = 0; a < n_rt; ++a) bl += wts[a] * env[(er + a) * ew];
        f3 x = ld3(cb + size_t(cb_row[i]) * cbw);
        f3 g;
        const float z = membrane_depth(x, ld3(cc + 3 * size_t(cc_row[i])), P.curved, P.sign, g);
        float sl, dsl;
        csig(z - P.lr_node, P.lr_sharp, sl, dsl);
        const float ll = sl, lr = 1.f - sl, dll = dsl, dlr = -dsl;
        const float cl = (z - P.z0) * P.zs, cr = (-z - P.z0) * P.zs;
        const float s_in = surf[size_t(s_row[i]) * sw];
        const bool outside = z > half || z < -half;
        const float* ci = coeff_in + size_t(rtype[i]) * P.n_node;
        float e = 0.f, dz = 0.f, dbl = 0.f, s2p = 0.f, ds2p = 0.f;
        for (int b = 0; b < n_bl; ++b) {
            float s1 = 1.f, ds1 = 0.f, s2 = 0.f, ds2 = 0.f;
            if (b < n_bl - 1) {
                float v, d;
                csig(bl - bl_nodes[b], P.bl_sharp, v, d);
                s1 = v; ds1 = d;
                csig(bl_nodes[b] - bl, P.bl_sharp, v, d);
                s2 = v; ds2 = -d;
            }
            float w, dw;
            if (b == 0) { w = s1; dw = ds1; }
            else if (b == n_bl - 1) { w = s2p; dw = ds2p; }
            else { w = s2p * s1; dw = ds2p * s1 + s2p * ds1; }
            s2p = s2;
            ds2p = ds2;
            const float sv = (b > 0 && outside) ? 1.f : s_in;
            const float* c = coeff + (size_t(rtype[i]) * n_bl + b) * P.n_node;
            float v, dv;
            clamped(c, cl, P.n_node, v, dv);
            float fl = v * sv, dfl = dv * P.zs * sv;
            clamped(c, cr, P.n_node, v, dv);
            float fr = v * sv, dfr = -dv * sv * P.zs;
            if (sv < 1.f) {
                clamped(ci, cl, P.n_node, v, dv);
                fl += v * (1.f - sv);
                dfl += dv * (1.f - sv) * P.zs;
                clamped(ci, cr, P.n_node, v, dv);
                fr += v * (1.f - sv);
                dfr -= dv * (1.f - sv) * P.zs;
            }
            const float fs = ll * fl + lr * fr, dfs = ll * dfl + dll * fl + lr * dfr + dlr * fr;
            e += w * fs;
            dbl += dw * fs;
            dz += w * dfs;
        }
        add_energy(pot, sys[i], e);
        atomic_add3(cbs + size_t(cb_row[i]) * cbw, g * dz);
        for (int a = 0; a < n_rt; ++a) atomicAdd(envs + (er + a) * ew, wts[a] * dbl);
    }
}
// backbone H/O term with the surface score (MembraneSurfHBPotential,
// src/membrane_potential.cpp:989-1259): the bonded / free depth splines
// weighted by outer = s * compact_sigmoid(burial - 2.5, 2) of the residue,
// the inner tables by 1 - outer (s = 1 outside the slab)
__global__ void memb_surf_hb_kernel(int n, MembParams P, float half, int n_rt, const int* __restrict__ hb_row,
                                    const int* __restrict__ env_row, const int* __restrict__ cc_row,
                                    const int* __restrict__ s_row, const int* __restrict__ htype,
                                    const int* __restrict__ sys, const float* __restrict__ wts,
                                    const float* __restrict__ coeff, const float* __restrict__ coeff_in, int hw,
                                    const float* __restrict__ hb, float* hbs, int ew, const float* __restrict__ env,
                                    float* envs, int sw, const float* __restrict__ surf, const float* __restrict__ cc,
                                    double* pot) {
    grid_dep_entry();
    for (int i = grid_stride_start(); i < n; i += grid_stride()) {
        const float* r = hb + size_t(hb_row[i]) * hw;
        f3 g;
        const float z = membrane_depth(ld3(r), ld3(cc + 3 * size_t(cc_row[i])), P.curved, P.sign, g);
        const size_t er = size_t(env_row[i]);
        float bl = 0.f;
        for (int a = 0; a < n_rt; ++a) bl += wts[a] * env[(er + a) * ew];
        float sb, dsb;
        csig(bl - 2.5f, 2.f, sb, dsb);
        float sv = surf[size_t(s_row[i]) * sw];
        if (z > half || z < -half) sv = 1.f;
        const float outer = sv * sb, d_outer = sv * dsb, inner = 1.f - outer, d_inner = -d_outer;
        const float u = 1.f - r[6], w1 = u * u, w2 = 1.f - w1;
        float e = 0.f, dZ = 0.f, dHB = 0.f, dBL = 0.f;
        for (int part = 0; part < 2; ++part) {
            const float wgt = part == 0 ? outer : inner, dwgt = part == 0 ? d_outer : d_inner;
            if (!(wgt > 0.f)) continue;
            const float* c = (part == 0 ? coeff : coeff_in) + size_t(htype[i]) * 2 * P.n_node;
            float f1, df1, f2, df2;
            mirrored_spline(c, P.n_node, z, P.z0, P.zs, P.lr_node, P.lr_sharp, f1, df1);
            mirrored_spline(c + P.n_node, P.n_node, z, P.z0, P.zs, P.lr_node, P.lr_sharp, f2, df2);
            e += w1 * wgt * f1 + w2 * wgt * f2;
            dHB += -2.f * u * wgt * f1 + 2.f * u * wgt * f2;
            dBL += w1 * dwgt * f1 + w2 * dwgt * f2;
            dZ += w1 * wgt * df1 + w2 * wgt * df2;
        }
        add_energy(pot, sys[i], e);
        float* rs = hbs + size_t(hb_row[i]) * hw;
        atomicAdd(rs + 6, dHB);
        atomic_add3(rs, g * dZ);
        for (int a = 0; a < n_rt; ++a) atomicAdd(envs + (er + a) * ew, wts[a] * dBL);
    }
}
// lateral pressure (MembraneLateralPotential, src/membrane_potential.cpp:
// 1262-1354): a force, no energy, of s * p((z - min_z) * inv_dz) *
// compact_sigmoid(burial - midpoint, sharpness) against the residue's surface
// force direction, p the clamped spline of the pressure profile
__global__ void lateral_kernel(int n, float half, float min_z, float inv_dz, int n_knot, const int* __restrict__ cb_row,
                               const int* __restrict__ env_row, const int* __restrict__ s_row,
                               const int* __restrict__ rtype, const float* __restrict__ wts,
                               const float* __restrict__ mid, const float* __restrict__ sharp,
                               const float* __restrict__ params, int cbw, const float* __restrict__ cb, float* cbs, int ew,
                               const float* __restrict__ env, int sw, const float* __restrict__ surf) {
    grid_dep_entry();
    for (int i = grid_stride_start(); i < n; i += grid_stride()) {
        const float z = cb[size_t(cb_row[i]) * cbw + 2];
        const float* sr = surf + size_t(s_row[i]) * sw;
        float sv = sr[0];
        if (z > half || z < -half) sv = 1.f;
        const size_t er = size_t(env_row[i]);
        float wbl = 0.f;
        for (int a = 0; a < 20; ++a) wbl += wts[a] * env[(er + a) * ew];
        const int t = rtype[i];
        float cs, dcs;
        csig(wbl - mid[t], sharp[t], cs, dcs);
        if (sv <= 0.f || cs == 0.f) continue;
        float v, dv;
        clamped(params, (z - min_z) * inv_dz, n_knot, v, dv);
        const float fm = sv * v;
        float* o = cbs + size_t(cb_row[i]) * cbw;
        atomicAdd(o, -(fm * cs * sr[1]));
        atomicAdd(o + 1, -(fm * cs * sr[2]));
    }
}

// cb_surf_membrane_potential: arguments (CB points, environment coverage,
// surface, curvature centre); hb_surf_membrane_potential: (protein_hbond,
// environment coverage, surface, curvature centre)
struct MembraneSurfNode : GNode {
    bool cb_term;
    int n = 0, n_rt = 0, n_bl = 1;
    float half = 0.f;
    MembParams P{};
    int *row = nullptr, *env_row = nullptr, *cc_row = nullptr, *s_row = nullptr, *type = nullptr, *sysv = nullptr;
    float *wts = nullptr, *bl_nodes = nullptr, *coeff = nullptr, *coeff_in = nullptr;
    std::vector<float> h_coeff;
    MembraneSurfNode(Engine& e, const Groups& g, bool cb, const GNode& pts, const GNode& env, const GNode& surf,
                     const GNode& cc)
        : cb_term(cb) {
        potential = true;
        const char* idx = cb ? "cb_index" : "hb_index";
        auto so = offsets(counts(g, idx));
        n = so.back();
        if (pts.width < (cb ? 3 : 7)) throw Error(cb ? "CB coordinates need width 3" : "protein_hbond needs width 7");
        if (surf.width < 1) throw Error("surface needs width 1");
        auto d = g.f(0).dims(g.p("coeff"));
        auto di = g.f(0).dims(g.p("coeff_inner"));
        if (d.size() != 3) throw Error("coeff must be 3-dimensional");
        h_coeff = shared_f(g, "coeff");
        P.n_node = int(d[2]);
        if (P.n_node < 4) throw Error("coeff needs at least 4 nodes");
        P.z0 = float(shared_attr(g, "z_start"));
        P.zs = float(shared_attr(g, "z_scale"));
        P.lr_node = float(shared_attr(g, "left_right_node"));
        P.lr_sharp = float(shared_attr(g, "left_right_sharpness"));
        P.curved = int(shared_attr(g, "use_curvature"));
        P.sign = float(shared_attr(g, "curvature_sign"));
        half = float(shared_attr(g, "half_thickness"));
        auto w = shared_f(g, "weights");
        if (cb) {
            n_rt = int(d[0]);
            n_bl = int(d[1]);
            if (di.size() != 2 || int(di[0]) != n_rt || int(di[1]) != P.n_node)
                throw Error("coeff_inner must be (n_restype, n_node)");
            if (int(w.size()) < n_rt) throw Error("weights needs one entry per residue type");
            P.bl_sharp = float(shared_attr(g, "bl_range_sharpness"));
            auto bn = shared_f(g, "bl_nodes");
            if (int(bn.size()) != n_bl - 1 || n_bl < 2) throw Error("bl_nodes must have n_bl - 1 entries");
            bl_nodes = e.upload(bn);
        } else {
            if (d[0] != 2 || d[1] != 2) throw Error("coeff must be (2, 2, n_node)");
            if (di.size() != 3 || di[0] != 2 || di[1] != 2 || int(di[2]) != P.n_node)
                throw Error("coeff_inner must be (2, 2, n_node)");
            n_rt = int(w.size());
        }
        wts = e.upload(w);
        coeff_in = e.upload(shared_f(g, "coeff_inner"));
        auto rows = cat_rows(g, idx, pts.off);
        std::vector<int> ty, ccr, envr, sr;
        for (size_t s = 0; s < g.size(); ++s) {
            if (cc.off[s + 1] - cc.off[s] < 1) throw Error("curvature centre has no row");
            auto types = read_i(g.f(s), g.p(cb ? "res_type" : "hb_type"));
            auto res = cb ? read_i(g.f(s), g.p(idx)) : read_i(g.f(s), g.p("hb_res"));
            const int m = so[s + 1] - so[s];
            if (int(types.size()) != m || int(res.size()) != m)
                throw Error(std::string(cb ? "res_type" : "hb_type and hb_res") + " need one entry per index");
            const int elim = env.off[s + 1] - env.off[s], slim = surf.off[s + 1] - surf.off[s];
            for (int i = 0; i < m; ++i) {
                const int t = types[size_t(i)], r = res[size_t(i)];
                if (t < 0 || t >= (cb ? n_rt : 2)) throw Error("type out of range");
                if (r < 0 || (r + 1) * n_rt > elim) throw Error("environment coverage has no row for residue " + std::to_string(r));
                if (r >= slim) throw Error("surface has no row for residue " + std::to_string(r));
                ty.push_back(t);
                envr.push_back(env.off[s] + r * n_rt);
                sr.push_back(surf.off[s] + r);
                ccr.push_back(cc.off[s]);
            }
        }
        row = e.upload(rows);
        env_row = e.upload(envr);
        s_row = e.upload(sr);
        cc_row = e.upload(ccr);
        type = e.upload(ty);
        sysv = e.upload(sys_of(so));
        coeff = e.upload(h_coeff);
    }
    void forward(Engine& e, bool energy) override {
        double* pot = energy ? e.d_pot + size_t(pot_slot) * e.n_sys : nullptr;
        auto &pts = e.arg(*this, 0), &env = e.arg(*this, 1), &sf = e.arg(*this, 2), &cc = e.arg(*this, 3);
        if (cb_term)
            ug::launch(memb_surf_cb_kernel, nblk(n), 256, 0, e.st, n, P, half, n_rt, n_bl, row, env_row, cc_row, s_row,
                       type, sysv, wts, bl_nodes, coeff, coeff_in, pts.width, pts.out, pts.sens, env.width, env.out,
                       env.sens, sf.width, sf.out, cc.out, pot);
        else
            ug::launch(memb_surf_hb_kernel, nblk(n), 256, 0, e.st, n, P, half, n_rt, row, env_row, cc_row, s_row, type,
                       sysv, wts, coeff, coeff_in, pts.width, pts.out, pts.sens, env.width, env.out, env.sens, sf.width,
                       sf.out, cc.out, pot);
    }
    // the outer spline coefficients (get_param / set_param of the reference node)
    std::vector<float> get_param(Engine&) override { return h_coeff; }
    void set_param(Engine& e, const std::vector<float>& p) override {
        if (p.size() != h_coeff.size()) throw Error("the size of parameters should be " + std::to_string(h_coeff.size()));
        h_coeff = p;
        UG_CK(cudaMemcpyAsync(coeff, h_coeff.data(), 4 * h_coeff.size(), cudaMemcpyHostToDevice, e.st));
        UG_CK(cudaStreamSynchronize(e.st));
    }
};

// membranelateral_potential: arguments (CB points, environment coverage,
// surface).  The reference reads the residue type and the weighted burial of
// entry i at index cb_index[i] (src/membrane_potential.cpp:1332-1336), so every
// cb_index entry must be below the number of entries.
struct LateralNode : GNode {
    int n = 0, n_knot = 0;
    float half = 0.f, min_z = 0.f, inv_dz = 0.f;
    int *cb_row = nullptr, *env_row = nullptr, *s_row = nullptr, *type = nullptr;
    float *wts = nullptr, *mid = nullptr, *sharp = nullptr, *params = nullptr;
    LateralNode(Engine& e, const Groups& g, const GNode& pts, const GNode& env, const GNode& surf) {
        potential = true;
        if (pts.width < 3) throw Error("CB coordinates need width 3");
        if (surf.width < 3) throw Error("surface needs width 3");
        half = float(shared_attr(g, "half_thickness"));
        min_z = float(shared_attr(g, "min_z"));
        inv_dz = float(shared_attr(g, "inv_dz"));
        n_knot = int(shared_attr(g, "n_knot"));
        auto w = shared_f(g, "weights"), m = shared_f(g, "cov_midpoint"), sh = shared_f(g, "cov_sharpness"),
             pp = shared_f(g, "params");
        if (w.size() != 20 || m.size() != 20 || sh.size() != 20)
            throw Error("weights, cov_midpoint and cov_sharpness need 20 entries");
        if (int(pp.size()) != n_knot || n_knot < 4) throw Error("params needs n_knot (at least 4) entries");
        std::vector<int> cr, er, sr, ty;
        for (size_t s = 0; s < g.size(); ++s) {
            auto ci = read_i(g.f(s), g.p("cb_index"));
            auto rt = read_i(g.f(s), g.p("restypes"));
            const int m_ = int(ci.size());
            if (int(rt.size()) != m_) throw Error("restypes needs one entry per cb_index");
            const int plim = pts.off[s + 1] - pts.off[s], elim = env.off[s + 1] - env.off[s],
                      slim = surf.off[s + 1] - surf.off[s];
            if (m_ * 20 > elim) throw Error("environment coverage has fewer than 20 rows per entry");
            for (int i = 0; i < m_; ++i) {
                const int r = ci[size_t(i)];
                if (r < 0 || r >= m_) throw Error("cb_index entries must be below the number of entries");
                if (r >= plim || r >= slim) throw Error("no CB or surface row for residue " + std::to_string(r));
                if (rt[size_t(r)] < 0 || rt[size_t(r)] >= 20) throw Error("restypes out of range");
                cr.push_back(pts.off[s] + r);
                er.push_back(env.off[s] + 20 * r);
                sr.push_back(surf.off[s] + r);
                ty.push_back(rt[size_t(r)]);
            }
        }
        n = int(cr.size());
        cb_row = e.upload(cr.empty() ? std::vector<int>(1, 0) : cr);
        env_row = e.upload(er.empty() ? std::vector<int>(1, 0) : er);
        s_row = e.upload(sr.empty() ? std::vector<int>(1, 0) : sr);
        type = e.upload(ty.empty() ? std::vector<int>(1, 0) : ty);
        wts = e.upload(w);
        mid = e.upload(m);
        sharp = e.upload(sh);
        params = e.upload(pp);
    }
    void forward(Engine& e, bool) override {
        auto &pts = e.arg(*this, 0), &env = e.arg(*this, 1), &sf = e.arg(*this, 2);
        if (n == 0) return;
        ug::launch(lateral_kernel, nblk(n), 256, 0, e.st, n, half, min_z, inv_dz, n_knot, cb_row, env_row, s_row, type,
                   wts, mid, sharp, params, pts.width, pts.out, pts.sens, env.width, env.out, sf.width, sf.out);
    }
};
