// Learned BP warm start: device state and launchers (warm.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ug {

constexpr int WARM_IN = 64;    // features per residue (51 used, zero-padded)
constexpr int WARM_HID = 128;  // hidden width of both layers
constexpr int WARM_OUT = 8;    // rotamer logits (6 used)
// every WARM_PROBE-th solve of a system tries the start it does not use, to
// keep measuring whether the learned start pays
constexpr int WARM_PROBE = 64;

// Whether a system's next BP solve starts from the warm start, from its sweep
// statistics ws = (mean sweeps warm, mean sweeps uniform, solves, known bits:
// 1 warm mean set, 2 uniform mean set).  The first solve measures the uniform
// start, the second the warm one; after that the warm start is used only
// while it saves at least WARM_MIN_GAIN sweeps, the price of the network: its
// feature and MLP kernels sit on the rotamer node's critical path and cost
// about as much device time as ten BP sweeps (measured on 64 systems of
// 40-400 residues: 0.13 ms per force evaluation against 13 us per sweep).
// Every WARM_PROBE-th solve tries the other start.  A start that runs no
// kernels of its own (the previous solve's marginals) needs to save only
// WARM_MIN_GAIN_FREE sweeps.
constexpr float WARM_MIN_GAIN = 8.f;
constexpr float WARM_MIN_GAIN_FREE = 0.5f;
__host__ __device__ inline bool warm_start_used(const float* ws, float min_gain = WARM_MIN_GAIN) {
    int solves = int(ws[2]), known = int(ws[3]);
    bool prefer_warm = (known & 2) != 0 && ((known & 1) == 0 || ws[0] + min_gain <= ws[1]);
    bool probe = (known & 3) == 3 && solves % WARM_PROBE == WARM_PROBE - 1;
    return prefer_warm != probe;
}

struct WarmDev {
    int* need;             // device flag: some system starts from the prediction in this solve
                           // (set by the features kernel)
    const float* stat;     // per-system sweep statistics (4 floats each)
    int n_sys;
    const int* node_res;   // BP node -> chain residue index within its system
    const int* node_aa;    // BP node -> residue type 0..19 (-1 unknown)
    int max_chain;         // largest chain length (residues) of one system
    uint16_t* X;           // n_node x WARM_IN features, bf16
    const uint16_t* W1;    // WARM_IN x WARM_HID, bf16, row-major
    const float* b1;
    const uint16_t* W2;    // WARM_HID x WARM_HID
    const float* b2;
    const uint16_t* W3;    // WARM_HID x WARM_OUT
    const float* b3;
    float* belief;         // n_node x 8 predicted marginals
};

// features only (for training data) or features + network + softmax
void launch_warm_features(const WarmDev& w, const float* pos, const int* atom_off, const int* res_off,
                          const float* prob, const int* nrot, int n_sys, cudaStream_t st);
cudaError_t launch_warm_start(const WarmDev& w, const float* pos, const int* atom_off, const int* res_off,
                              const float* prob, const int* nrot, int n_sys, int n_res, cudaStream_t st);

// training and inference building blocks (bf16 operands, FP32 accumulation)
// need: optional device flag; when it reads 0 the kernel does nothing
cudaError_t launch_gemm_bf16(const uint16_t* A, long long a_r, long long a_c, const uint16_t* B, long long b_r,
                             long long b_c, float* C, int ldc, int M, int N, int K, int accumulate, cudaStream_t st,
                             const int* need = nullptr);
cudaError_t launch_bias_act(const float* Z, const float* bias, uint16_t* H, float* Hf, int M, int N, int relu,
                            cudaStream_t st, const int* need = nullptr);
cudaError_t launch_to_bf16(float* X, const uint16_t* H, uint16_t* Y, long long n, cudaStream_t st);
cudaError_t launch_softmax_xent(const float* Z, const float* T, const int* nrot, float* dZ, float* loss, int M,
                                float scale, cudaStream_t st);
cudaError_t launch_colsum(const float* X, float* out, int M, int N, cudaStream_t st);
cudaError_t launch_adam(float* w, const float* g, float* m, float* v, uint16_t* wb, int n, float lr, float b1, float b2,
                        float eps, int step, cudaStream_t st);

}  // namespace ug
