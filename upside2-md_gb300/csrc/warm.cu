// Learned warm start for the rotamer BP solve: per-residue geometric
// features, a small bf16 MLP (features -> 128 -> 128 -> 8 rotamer logits,
// FP32 accumulation) and its training kernels.
//
// The MLP predicts each residue's converged rotamer marginal from its local
// geometry; the BP solve starts from that prediction instead of the
// one-body probabilities (src/rotamer.cpp:1110-1135 is the uniform start it
// replaces).  BP still iterates to the reference's tolerance, so the network
// only changes where the iteration starts.
//
// GEMMs use the warp-level tensor-core instruction mma.sync m16n8k16 (bf16
// in, FP32 accumulate): the network is ~25k parameters and its GEMMs are
// (residues x 64..128) x (64..128 x 128), far below a tile schedule that
// would need the tcgen05/TMEM path.
#include <cstdint>

#include "dev_math.cuh"
#include "launch.cuh"
#include "warm.h"

namespace ug {

// ------------------------------------------------------------------ bf16 --
// round-to-nearest-even FP32 -> bf16 and back, by bit manipulation (finite
// inputs; NaN is kept a NaN)
__device__ __forceinline__ uint16_t f2bf(float x) {
    uint32_t u = __float_as_uint(x);
    if ((u & 0x7f800000u) == 0x7f800000u) return uint16_t((u >> 16) | ((u & 0xffffu) ? 0x40u : 0u));
    u += 0x7fffu + ((u >> 16) & 1u);
    return uint16_t(u >> 16);
}
__device__ __forceinline__ float bf2f(uint16_t h) { return __uint_as_float(uint32_t(h) << 16); }

// --------------------------------------------------------------- GEMM ---
// C[M x N] (FP32, row-major, ldc) (+)= A[M x K] . B[K x N] with A(i,k) at
// A[i*a_r + k*a_c] and B(k,n) at B[k*b_r + n*b_c] (bf16), so any operand can
// be a transpose.  Block tile 64 x 64, K step 32, 4 warps of 32 x 32; the
// tiles are staged through shared memory in the fragment-friendly layouts
// (A row-major, B n-major) and multiplied with mma.sync m16n8k16.
constexpr int GT_M = 64, GT_N = 64, GT_K = 32;

__device__ __forceinline__ uint32_t pack2(uint16_t lo, uint16_t hi) { return uint32_t(lo) | (uint32_t(hi) << 16); }

__global__ void __launch_bounds__(128) gemm_bf16_kernel(const uint16_t* __restrict__ A, long long a_r, long long a_c,
                                                        const uint16_t* __restrict__ B, long long b_r, long long b_c,
                                                        float* __restrict__ C, int ldc, int M, int N, int K,
                                                        int accumulate, const int* __restrict__ need) {
    grid_dep_entry();
    if (need && !*need) return;  // block-uniform: nothing to compute this time
    __shared__ uint16_t As[GT_M][GT_K + 8];  // [m][k]
    __shared__ uint16_t Bs[GT_N][GT_K + 8];  // [n][k]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int m0 = blockIdx.y * GT_M, n0 = blockIdx.x * GT_N;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;  // warp tile origin in the block tile
    const int g = lane >> 2, t = lane & 3;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;

    for (int k0 = 0; k0 < K; k0 += GT_K) {
        for (int x = tid; x < GT_M * GT_K; x += 128) {
            int mi = x / GT_K, ki = x % GT_K;
            int gm = m0 + mi, gk = k0 + ki;
            As[mi][ki] = (gm < M && gk < K) ? A[gm * a_r + gk * a_c] : uint16_t(0);
        }
        for (int x = tid; x < GT_N * GT_K; x += 128) {
            int ni = x / GT_K, ki = x % GT_K;
            int gn = n0 + ni, gk = k0 + ki;
            Bs[ni][ki] = (gn < N && gk < K) ? B[gk * b_r + gn * b_c] : uint16_t(0);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GT_K; kk += 16) {
            uint32_t af[2][4], bfr[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                int r = wm + i * 16 + g;
                af[i][0] = pack2(As[r][kk + 2 * t], As[r][kk + 2 * t + 1]);
                af[i][1] = pack2(As[r + 8][kk + 2 * t], As[r + 8][kk + 2 * t + 1]);
                af[i][2] = pack2(As[r][kk + 2 * t + 8], As[r][kk + 2 * t + 9]);
                af[i][3] = pack2(As[r + 8][kk + 2 * t + 8], As[r + 8][kk + 2 * t + 9]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                int c = wn + j * 8 + g;
                bfr[j][0] = pack2(Bs[c][kk + 2 * t], Bs[c][kk + 2 * t + 1]);
                bfr[j][1] = pack2(Bs[c][kk + 2 * t + 8], Bs[c][kk + 2 * t + 9]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    asm volatile(
                        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
                        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                        : "+f"(acc[i][j][0]), "+f"(acc[i][j][1]), "+f"(acc[i][j][2]), "+f"(acc[i][j][3])
                        : "r"(af[i][0]), "r"(af[i][1]), "r"(af[i][2]), "r"(af[i][3]), "r"(bfr[j][0]),
                          "r"(bfr[j][1]));
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                int row = m0 + wm + i * 16 + g + (r >= 2 ? 8 : 0);
                int col = n0 + wn + j * 8 + 2 * t + (r & 1);
                if (row < M && col < N) {
                    float* c = C + size_t(row) * ldc + col;
                    *c = accumulate ? *c + acc[i][j][r] : acc[i][j][r];
                }
            }
}

cudaError_t launch_gemm_bf16(const uint16_t* A, long long a_r, long long a_c, const uint16_t* B, long long b_r,
                             long long b_c, float* C, int ldc, int M, int N, int K, int accumulate, cudaStream_t st,
                             const int* need) {
    if (M <= 0 || N <= 0) return cudaSuccess;
    dim3 grid((N + GT_N - 1) / GT_N, (M + GT_M - 1) / GT_M);
    ug::launch(gemm_bf16_kernel, grid, 128, 0, st, A, a_r, a_c, B, b_r, b_c, C, ldc, M, N, K, accumulate, need);
    return cudaGetLastError();
}

// ---------------------------------------------------------- epilogues ---
// H = bf16(act(Z + bias)), act = ReLU or identity
__global__ void bias_act_kernel(const float* __restrict__ Z, const float* __restrict__ bias, uint16_t* __restrict__ H,
                                float* __restrict__ Hf, int M, int N, int relu, const int* __restrict__ need) {
    grid_dep_entry();
    if (need && !*need) return;
    long long n = (long long)M * N;
    for (long long i = grid_stride_start(); i < n; i += grid_stride()) {
        float v = Z[i] + bias[i % N];
        if (relu) v = fmaxf(v, 0.f);
        if (H) H[i] = f2bf(v);
        if (Hf) Hf[i] = v;
    }
}

// FP32 -> bf16 copy.  With H given, the ReLU derivative of the forward
// activation is applied first (dZ = dH where H > 0) and the masked FP32
// value is written back into X too (for the bias gradient).
__global__ void to_bf16_kernel(float* __restrict__ X, const uint16_t* __restrict__ H, uint16_t* __restrict__ Y,
                               long long n) {
    grid_dep_entry();
    for (long long i = grid_stride_start(); i < n; i += grid_stride()) {
        float v = X[i];
        if (H && !(bf2f(H[i]) > 0.f)) {
            v = 0.f;
            X[i] = 0.f;
        }
        Y[i] = f2bf(v);
    }
}

// Softmax cross-entropy against soft targets over the first n_rot of
// WARM_OUT logits per row (rows with n_rot < 2 carry no loss):
// dlogits = (softmax - target) / n_rows_with_loss, loss summed into *loss.
__global__ void softmax_xent_kernel(const float* __restrict__ Z, const float* __restrict__ T,
                                    const int* __restrict__ nrot, float* __restrict__ dZ, float* __restrict__ loss,
                                    int M, float scale) {
    grid_dep_entry();
    for (int i = grid_stride_start(); i < M; i += grid_stride()) {
        int n = nrot[i];
        const float* z = Z + size_t(i) * WARM_OUT;
        float* d = dZ + size_t(i) * WARM_OUT;
        if (n < 2) {
            for (int k = 0; k < WARM_OUT; ++k) d[k] = 0.f;
            continue;
        }
        float mx = z[0];
        for (int k = 1; k < n; ++k) mx = fmaxf(mx, z[k]);
        float p[WARM_OUT], s = 0.f;
        for (int k = 0; k < WARM_OUT; ++k) {
            p[k] = k < n ? expf(z[k] - mx) : 0.f;
            s += p[k];
        }
        float l = 0.f, ls = logf(s);
        for (int k = 0; k < WARM_OUT; ++k) {
            float t = k < n ? T[size_t(i) * WARM_OUT + k] : 0.f;
            float pk = p[k] / s;
            d[k] = k < n ? (pk - t) * scale : 0.f;
            if (k < n && t > 0.f) l -= t * (z[k] - mx - ls);
        }
        atomicAdd(loss, l * scale);
    }
}

// column sums of X[M x N] (bias gradients)
__global__ void colsum_kernel(const float* __restrict__ X, float* __restrict__ out, int M, int N) {
    grid_dep_entry();
    int c = blockIdx.x;
    float s = 0.f;
    for (int r = threadIdx.x; r < M; r += blockDim.x) s += X[size_t(r) * N + c];
    __shared__ float red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = red[0];
}

// Adam on FP32 master weights; the bf16 copy used by the GEMMs is refreshed
__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, uint16_t* __restrict__ wb, int n, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
    grid_dep_entry();
    for (int i = grid_stride_start(); i < n; i += grid_stride()) {
        float gi = g[i];
        float mi = b1 * m[i] + (1.f - b1) * gi;
        float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
        w[i] = wi;
        if (wb) wb[i] = f2bf(wi);
    }
}

static int nb(long long n) { return int(std::min<long long>(4 * 152, (n + 255) / 256)); }

cudaError_t launch_bias_act(const float* Z, const float* bias, uint16_t* H, float* Hf, int M, int N, int relu,
                            cudaStream_t st, const int* need) {
    ug::launch(bias_act_kernel, nb((long long)M * N), 256, 0, st, Z, bias, H, Hf, M, N, relu, need);
    return cudaGetLastError();
}
cudaError_t launch_to_bf16(float* X, const uint16_t* H, uint16_t* Y, long long n, cudaStream_t st) {
    ug::launch(to_bf16_kernel, nb(n), 256, 0, st, X, H, Y, n);
    return cudaGetLastError();
}
cudaError_t launch_softmax_xent(const float* Z, const float* T, const int* nrot, float* dZ, float* loss, int M,
                                float scale, cudaStream_t st) {
    ug::launch(softmax_xent_kernel, nb(M), 256, 0, st, Z, T, nrot, dZ, loss, M, scale);
    return cudaGetLastError();
}
cudaError_t launch_colsum(const float* X, float* out, int M, int N, cudaStream_t st) {
    if (N <= 0) return cudaSuccess;
    ug::launch(colsum_kernel, N, 256, 0, st, X, out, M, N);
    return cudaGetLastError();
}
cudaError_t launch_adam(float* w, const float* g, float* m, float* v, uint16_t* wb, int n, float lr, float b1, float b2,
                        float eps, int step, cudaStream_t st) {
    float c1 = 1.f / (1.f - powf(b1, float(step))), c2 = 1.f / (1.f - powf(b2, float(step)));
    ug::launch(adam_kernel, nb(n), 256, 0, st, w, g, m, v, wb, n, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError();
}

// ---------------------------------------------------------- features ---
// Virtual C-beta from the backbone (the ideal-geometry construction used by
// trRosetta-style structure featurisers: a fixed combination of the N-CA and
// CA-C bond vectors and their cross product).
__device__ __forceinline__ f3 virtual_cb(f3 n, f3 ca, f3 c) {
    f3 b = ca - n, cc = c - ca;
    f3 a = cross(b, cc);
    return a * -0.58273431f + b * 0.56802827f - cc * 0.54067466f + ca;
}

__device__ __forceinline__ float dihedral_angle(f3 p0, f3 p1, f3 p2, f3 p3) {
    f3 b0 = p1 - p0, b1 = p2 - p1, b2 = p3 - p2;
    f3 n1 = cross(b0, b1), n2 = cross(b1, b2);
    float x = dot(n1, n2);
    float y = dot(cross(n1, n2), b1) * rsqrtf(fmaxf(dot(b1, b1), 1e-12f));
    return atan2f(y, x);
}

// One block per system.  Backbone atoms of residue r are atoms 3r, 3r+1, 3r+2
// (N, CA, C) of the system.  Per BP node u (chain residue node_res[u]):
//   0-7    CA distances to residues r-4..r-1, r+1..r+4 (/10; 0 beyond the chain)
//   8-11   C-beta neighbour counts within 6, 8, 10, 12 A (/20)
//   12-13  half-sphere exposure: C-alphas within 13 A on the C-beta side / the other side (/20)
//   14-17  sin, cos of phi and psi (0, 1 at the termini)
//   18-21  sum of unit vectors to C-betas within 10 A in the residue frame (/10) and its norm (/10)
//   22     C-beta contacts within 8 A with sequence separation > 3 (/10)
//   23     1
//   24-43  residue type one-hot (20)
//   44-49  one-body log-probabilities of the node's rotamers, centred (/5, clipped to +-2)
//   50     1 if the node has 6 rotamers
//   51-63  0
__global__ void warm_features_kernel(WarmDev w, const float* __restrict__ pos, const int* __restrict__ atom_off,
                                     const int* __restrict__ res_off, const float* __restrict__ prob,
                                     const int* __restrict__ nrot) {
    grid_dep_entry();
    const int s = blockIdx.x;
    if (w.stat && w.need && blockIdx.x == 0 && blockIdx.y == 0) {
        // need = 1 when some system's coming solve starts from the prediction
        // (the statistics are final: the previous solve updated them); the
        // network's kernels read it after this kernel
        __shared__ int any;
        if (threadIdx.x == 0) any = 0;
        __syncthreads();
        for (int u = threadIdx.x; u < w.n_sys; u += blockDim.x)
            if (warm_start_used(w.stat + 4 * u)) any = 1;
        __syncthreads();
        if (threadIdx.x == 0) *w.need = any;
    }
    // only systems whose solve starts from the prediction need features
    if (w.stat && !warm_start_used(w.stat + 4 * s)) return;
    extern __shared__ float wsm[];
    const int a0 = atom_off[s], nres = (atom_off[s + 1] - a0) / 3;
    f3* CA = reinterpret_cast<f3*>(wsm);
    f3* CB = CA + nres;
    for (int r = threadIdx.x; r < nres; r += blockDim.x) {
        f3 n = ld3(pos + 3 * size_t(a0 + 3 * r)), ca = ld3(pos + 3 * size_t(a0 + 3 * r + 1)),
           c = ld3(pos + 3 * size_t(a0 + 3 * r + 2));
        CA[r] = ca;
        CB[r] = virtual_cb(n, ca, c);
    }
    __syncthreads();
    const int u0 = res_off[s], u1 = res_off[s + 1];
    // the system's nodes are spread over gridDim.y blocks
    for (int u = u0 + blockIdx.y * blockDim.x + threadIdx.x; u < u1; u += blockDim.x * gridDim.y) {
        if (nrot[u] == 1) {  // a single rotamer needs no prediction
            uint16_t* x = w.X + size_t(u) * WARM_IN;
            for (int k = 0; k < WARM_IN; ++k) x[k] = 0;
            continue;
        }
        float f[WARM_IN];
#pragma unroll
        for (int k = 0; k < WARM_IN; ++k) f[k] = 0.f;
        int r = w.node_res[u];
        f3 ca = CA[r], cb = CB[r];
#pragma unroll
        for (int k = 1; k <= 4; ++k) {
            f[4 - k] = r - k >= 0 ? sqrtf(mag2(CA[r - k] - ca)) * 0.1f : 0.f;
            f[3 + k] = r + k < nres ? sqrtf(mag2(CA[r + k] - ca)) * 0.1f : 0.f;
        }
        f3 e1 = cb - ca;
        e1 = e1 * rsqrtf(fmaxf(dot(e1, e1), 1e-12f));
        f3 nn = ld3(pos + 3 * size_t(a0 + 3 * r)), cc = ld3(pos + 3 * size_t(a0 + 3 * r + 2));
        f3 e2 = cc - nn;
        e2 = e2 - e1 * dot(e1, e2);
        e2 = e2 * rsqrtf(fmaxf(dot(e2, e2), 1e-12f));
        f3 e3 = cross(e1, e2);
        float c6 = 0.f, c8 = 0.f, c10 = 0.f, c12 = 0.f, up = 0.f, dn = 0.f, lr = 0.f;
        f3 acc = mk(0.f, 0.f, 0.f);
        for (int j = 0; j < nres; ++j) {
            if (j == r) continue;
            f3 d = CB[j] - cb;
            float d2 = dot(d, d);
            c6 += d2 < 36.f;
            c8 += d2 < 64.f;
            c10 += d2 < 100.f;
            c12 += d2 < 144.f;
            if (d2 < 100.f && d2 > 1e-6f) acc = acc + d * rsqrtf(d2);
            if (d2 < 64.f && abs(j - r) > 3) lr += 1.f;
            f3 v = CA[j] - ca;
            if (dot(v, v) < 169.f) {
                if (dot(v, e1) > 0.f) up += 1.f; else dn += 1.f;
            }
        }
        f[8] = c6 * 0.05f; f[9] = c8 * 0.05f; f[10] = c10 * 0.05f; f[11] = c12 * 0.05f;
        f[12] = up * 0.05f; f[13] = dn * 0.05f;
        float phi = 0.f, psi = 0.f;
        bool has_phi = r > 0, has_psi = r + 1 < nres;
        if (has_phi) phi = dihedral_angle(ld3(pos + 3 * size_t(a0 + 3 * r - 1)), nn, ca, cc);
        if (has_psi) psi = dihedral_angle(nn, ca, cc, ld3(pos + 3 * size_t(a0 + 3 * r + 3)));
        f[14] = has_phi ? sinf(phi) : 0.f; f[15] = has_phi ? cosf(phi) : 1.f;
        f[16] = has_psi ? sinf(psi) : 0.f; f[17] = has_psi ? cosf(psi) : 1.f;
        f[18] = dot(acc, e1) * 0.1f; f[19] = dot(acc, e2) * 0.1f; f[20] = dot(acc, e3) * 0.1f;
        f[21] = sqrtf(mag2(acc)) * 0.1f;
        f[22] = lr * 0.1f;
        f[23] = 1.f;
        int aa = w.node_aa[u];
        if (aa >= 0 && aa < 20) f[24 + aa] = 1.f;
        int n = nrot[u];
        float lp[6], mean = 0.f;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            lp[k] = k < n ? logf(fmaxf(prob[u * 8 + k], 1e-30f)) : 0.f;
            mean += k < n ? lp[k] : 0.f;
        }
        mean /= float(n);
#pragma unroll
        for (int k = 0; k < 6; ++k) f[44 + k] = k < n ? fminf(2.f, fmaxf(-2.f, (lp[k] - mean) * 0.2f)) : 0.f;
        f[50] = n == 6 ? 1.f : 0.f;
        uint16_t* x = w.X + size_t(u) * WARM_IN;
#pragma unroll
        for (int k = 0; k < WARM_IN; ++k) x[k] = f2bf(f[k]);
    }
}

void launch_warm_features(const WarmDev& w, const float* pos, const int* atom_off, const int* res_off,
                          const float* prob, const int* nrot, int n_sys, cudaStream_t st) {
    size_t smem = size_t(w.max_chain) * 2 * sizeof(f3);
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        cudaFuncSetAttribute(warm_features_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        configured = smem;
    }
    ug::launch(warm_features_kernel, dim3(unsigned(n_sys), 4), 128, smem, st, w, pos, atom_off, res_off, prob, nrot);
}

// The whole network for a tile of 64 residues in one block (4 warps, 16 rows
// each): the transposed weights are staged in shared memory once per block,
// each warp carries its rows through the three layers (its activations stay
// in its own 16 rows of one shared buffer) and finishes with the softmax over
// each residue's rotamers (the predicted marginals).  The K steps and the
// mma.sync shape are those of gemm_bf16_kernel (which the training path
// uses), in the same order.
constexpr int MLP_ROWS = 64;
constexpr int MLP_PAD = 8;  // bf16 row padding of the staged buffers (bank spread)
template <int NT>  // n-tiles of 8 columns
__device__ __forceinline__ void mlp_layer(const uint16_t* Hs, int hld, const uint16_t* Wt, int wld, int K, int row0,
                                          int g, int t, float (&acc)[NT][4]) {
#pragma unroll
    for (int j = 0; j < NT; ++j)
#pragma unroll
        for (int r = 0; r < 4; ++r) acc[j][r] = 0.f;
    for (int kk = 0; kk < K; kk += 16) {
        const int r = row0 + g;
        const uint32_t a0 = pack2(Hs[r * hld + kk + 2 * t], Hs[r * hld + kk + 2 * t + 1]);
        const uint32_t a1 = pack2(Hs[(r + 8) * hld + kk + 2 * t], Hs[(r + 8) * hld + kk + 2 * t + 1]);
        const uint32_t a2 = pack2(Hs[r * hld + kk + 2 * t + 8], Hs[r * hld + kk + 2 * t + 9]);
        const uint32_t a3 = pack2(Hs[(r + 8) * hld + kk + 2 * t + 8], Hs[(r + 8) * hld + kk + 2 * t + 9]);
#pragma unroll
        for (int j = 0; j < NT; ++j) {
            const int c = j * 8 + g;
            const uint32_t b0 = pack2(Wt[c * wld + kk + 2 * t], Wt[c * wld + kk + 2 * t + 1]);
            const uint32_t b1 = pack2(Wt[c * wld + kk + 2 * t + 8], Wt[c * wld + kk + 2 * t + 9]);
            asm volatile(
                "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
                "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                : "+f"(acc[j][0]), "+f"(acc[j][1]), "+f"(acc[j][2]), "+f"(acc[j][3])
                : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
        }
    }
}
__global__ void __launch_bounds__(128) warm_mlp_kernel(WarmDev w, const int* __restrict__ nrot, int n_res) {
    grid_dep_entry();
    if (w.need && !*w.need) return;  // block-uniform: no system starts from the prediction
    extern __shared__ uint16_t mlp_sm[];
    constexpr int LD_IN = WARM_IN + MLP_PAD, LD_HID = WARM_HID + MLP_PAD;
    uint16_t* W1t = mlp_sm;                        // [WARM_HID][LD_IN]
    uint16_t* W2t = W1t + WARM_HID * LD_IN;        // [WARM_HID][LD_HID]
    uint16_t* W3t = W2t + WARM_HID * LD_HID;       // [WARM_OUT][LD_HID]
    uint16_t* Xs = W3t + WARM_OUT * LD_HID;        // [MLP_ROWS][LD_IN]
    uint16_t* Hs = Xs + MLP_ROWS * LD_IN;          // [MLP_ROWS][LD_HID]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, g = lane >> 2, t = lane & 3;
    for (int x = tid; x < WARM_IN * WARM_HID; x += 128) {  // W1 is [k][n]
        const int k = x / WARM_HID, n = x % WARM_HID;
        W1t[n * LD_IN + k] = w.W1[x];
    }
    for (int x = tid; x < WARM_HID * WARM_HID; x += 128) {
        const int k = x / WARM_HID, n = x % WARM_HID;
        W2t[n * LD_HID + k] = w.W2[x];
    }
    for (int x = tid; x < WARM_HID * WARM_OUT; x += 128) {
        const int k = x / WARM_OUT, n = x % WARM_OUT;
        W3t[n * LD_HID + k] = w.W3[x];
    }
    const int m0 = blockIdx.x * MLP_ROWS;
    for (int x = tid; x < MLP_ROWS * WARM_IN; x += 128) {
        const int r = x / WARM_IN, k = x % WARM_IN;
        Xs[r * LD_IN + k] = m0 + r < n_res ? w.X[size_t(m0 + r) * WARM_IN + k] : uint16_t(0);
    }
    __syncthreads();
    const int row0 = warp * 16;
    float acc[WARM_HID / 8][4];
    // layer 1: relu(X . W1 + b1) -> this warp's rows of Hs
    mlp_layer(Xs, LD_IN, W1t, LD_IN, WARM_IN, row0, g, t, acc);
#pragma unroll
    for (int j = 0; j < WARM_HID / 8; ++j)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int row = row0 + g + (r >= 2 ? 8 : 0), col = j * 8 + 2 * t + (r & 1);
            Hs[row * LD_HID + col] = f2bf(fmaxf(acc[j][r] + w.b1[col], 0.f));
        }
    __syncwarp();
    // layer 2: relu(H1 . W2 + b2), written over the warp's own rows once read
    mlp_layer(Hs, LD_HID, W2t, LD_HID, WARM_HID, row0, g, t, acc);
    __syncwarp();
#pragma unroll
    for (int j = 0; j < WARM_HID / 8; ++j)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int row = row0 + g + (r >= 2 ? 8 : 0), col = j * 8 + 2 * t + (r & 1);
            Hs[row * LD_HID + col] = f2bf(fmaxf(acc[j][r] + w.b2[col], 0.f));
        }
    __syncwarp();
    // layer 3: H2 . W3 + b3 -> logits; softmax over the residue's rotamers
    float a3[1][4];
    mlp_layer(Hs, LD_HID, W3t, LD_HID, WARM_HID, row0, g, t, a3);
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        const int u = m0 + row0 + g + 8 * half;
        float z0 = a3[0][2 * half] + w.b3[2 * t], z1 = a3[0][2 * half + 1] + w.b3[2 * t + 1];
        // the residue's 8 logits from the 4 lanes of its quad, in order
        float z[8];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            z[2 * q] = __shfl_sync(0xffffffffu, z0, (lane & ~3) | q);
            z[2 * q + 1] = __shfl_sync(0xffffffffu, z1, (lane & ~3) | q);
        }
        if (u >= n_res || t != 0) continue;
        const int n = nrot[u];
        float mx = z[0];
        for (int k = 1; k < n; ++k) mx = fmaxf(mx, z[k]);
        float p[8], sum = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            p[k] = k < n ? expf(z[k] - mx) : 0.f;
            sum += p[k];
        }
        const float inv = 1.f / sum;
        float* b = w.belief + size_t(u) * 8;
#pragma unroll
        for (int k = 0; k < 8; ++k) b[k] = p[k] * inv;
    }
}
constexpr size_t warm_mlp_smem() {
    return sizeof(uint16_t) * (size_t(WARM_HID) * (WARM_IN + MLP_PAD) + size_t(WARM_HID) * (WARM_HID + MLP_PAD) +
                               size_t(WARM_OUT) * (WARM_HID + MLP_PAD) + size_t(MLP_ROWS) * (WARM_IN + MLP_PAD) +
                               size_t(MLP_ROWS) * (WARM_HID + MLP_PAD));
}

cudaError_t launch_warm_start(const WarmDev& w, const float* pos, const int* atom_off, const int* res_off,
                              const float* prob, const int* nrot, int n_sys, int n_res, cudaStream_t st) {
    // the features kernel sets need; when no system starts from the
    // prediction in this solve, every kernel after it returns at once
    launch_warm_features(w, pos, atom_off, res_off, prob, nrot, n_sys, st);
    // relu(X[n x 64] . W1[64 x 128] + b1) -> relu(. W2 + b2) -> . W3[128 x 8]
    // + b3 -> softmax over the rotamers, in one kernel
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(warm_mlp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(warm_mlp_smem()));
        configured = true;
    }
    if (n_res > 0)
        ug::launch(warm_mlp_kernel, (n_res + MLP_ROWS - 1) / MLP_ROWS, 128, warm_mlp_smem(), st, w, nrot, n_res);
    return cudaGetLastError();
}

}  // namespace ug
