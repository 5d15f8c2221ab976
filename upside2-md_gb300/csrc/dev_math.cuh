// Device math shared by the sm_103a kernels: small vector algebra, the
// clamped / periodic cubic B-splines, compact sigmoid.  FP32 throughout.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ug {

struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 mk(float a, float b, float c) { return f3{a, b, c}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ f3& operator+=(f3& a, f3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float mag2(f3 a) { return dot(a, a); }
__device__ __forceinline__ f3 ld3(const float* p) { return {p[0], p[1], p[2]}; }
__device__ __forceinline__ void st3(float* p, f3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }
__device__ __forceinline__ void atomic_add3(float* p, f3 v) {
    atomicAdd(p, v.x);
    atomicAdd(p + 1, v.y);
    atomicAdd(p + 2, v.z);
}

// compact sigmoid: 1 below -1/s, 0 above 1/s, cubic in between
__device__ __forceinline__ void csig(float x, float s, float& v, float& d) {
    float y = x * s;
    if (y > 1.f) { v = 0.f; d = 0.f; return; }
    if (y < -1.f) { v = 1.f; d = 0.f; return; }
    v = 0.25f * (y + 2.f) * (y - 1.f) * (y - 1.f);
    d = (s * 0.75f) * (y * y - 1.f);
}

__device__ __forceinline__ void logistic(float x, float& v, float& d) {
    float z = expf(-x);
    float w = 1.f / (1.f + z);
    v = w;
    d = z * w * w;
}

// uniform cubic B-spline weights on [0,1) and their derivatives
__device__ __forceinline__ void bsp4(float y, float b[4], float db[4]) {
    float y2 = y * y, y3 = y2 * y, o = 1.f - y;
    const float s6 = 1.f / 6.f;
    b[0] = o * o * o * s6;
    b[1] = (3.f * y3 - 6.f * y2 + 4.f) * s6;
    b[2] = (-3.f * y3 + 3.f * y2 + 3.f * y + 1.f) * s6;
    b[3] = y3 * s6;
    db[0] = -0.5f * o * o;
    db[1] = 1.5f * y2 - 2.f * y;
    db[2] = -1.5f * y2 + y + 0.5f;
    db[3] = 0.5f * y2;
}

// spline with the first basis centred at -1; x >= 1
__device__ __forceinline__ void deboor(const float* c, float x, float& v, float& d) {
    int xb = int(x);
    float b[4], db[4];
    bsp4(x - float(xb), b, db);
    const float* cc = c + (xb - 1);
    float c0 = cc[0], c1 = cc[1], c2 = cc[2], c3 = cc[3];
    v = c0 * b[0] + c1 * b[1] + c2 * b[2] + c3 * b[3];
    d = c0 * db[0] + c1 * db[1] + c2 * db[2] + c3 * db[3];
}

// clamped spline: constant continuation below x=1 and above x=n-2
__device__ __forceinline__ void clamped(const float* c, float x, int n, float& v, float& d) {
    if (x <= 1.f) {
        v = c[0] * (1.f / 6.f) + c[1] * (2.f / 3.f) + c[2] * (1.f / 6.f);
        d = 0.f;
    } else if (x >= float(n - 2)) {
        v = c[n - 3] * (1.f / 6.f) + c[n - 2] * (2.f / 3.f) + c[n - 1] * (1.f / 6.f);
        d = 0.f;
    } else {
        deboor(c, x, v, d);
    }
}

__device__ __forceinline__ int clamped_coeff_deriv(float x, int n, float r[4]) {
    if (x <= 1.f) { r[0] = 1.f / 6.f; r[1] = 2.f / 3.f; r[2] = 1.f / 6.f; r[3] = 0.f; return 0; }
    if (x >= float(n - 2)) { r[0] = 0.f; r[1] = 1.f / 6.f; r[2] = 2.f / 3.f; r[3] = 1.f / 6.f; return n - 4; }
    int xb = int(x);
    float db[4];
    bsp4(x - float(xb), r, db);
    return xb - 1;
}
__device__ __forceinline__ int coeff_deriv(float x, float r[4]) {
    int xb = int(x);
    float db[4];
    bsp4(x - float(xb), r, db);
    return xb - 1;
}

// Periodic bicubic B-spline over a (nx+3) x (ny+3) padded coefficient layer:
// padded[i][j] = C[(i-1) mod nx][(j-1) mod ny], so the 4x4 support of cell
// (xb, yb) is rows xb..xb+3, columns yb..yb+3 with no wrap-around.
__device__ __forceinline__ void periodic2d(const float* layer, int nyp, float x, float y, float& v, float& dx,
                                           float& dy) {
    int xb = int(x), yb = int(y);
    float bx[4], dbx[4], by[4], dby[4];
    bsp4(x - float(xb), bx, dbx);
    bsp4(y - float(yb), by, dby);
    v = dx = dy = 0.f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float* r = layer + (xb + i) * nyp + yb;
        float sv = r[0] * by[0] + r[1] * by[1] + r[2] * by[2] + r[3] * by[3];
        float sd = r[0] * dby[0] + r[1] * dby[1] + r[2] * dby[2] + r[3] * dby[3];
        v += bx[i] * sv;
        dx += dbx[i] * sv;
        dy += bx[i] * sd;
    }
}

__device__ __forceinline__ void quat_to_rot(const float* q, float* U) {
    float a = q[0], b = q[1], c = q[2], d = q[3];
    U[0] = a * a + b * b - c * c - d * d; U[1] = 2.f * b * c - 2.f * a * d; U[2] = 2.f * b * d + 2.f * a * c;
    U[3] = 2.f * b * c + 2.f * a * d; U[4] = a * a - b * b + c * c - d * d; U[5] = 2.f * c * d - 2.f * a * b;
    U[6] = 2.f * b * d - 2.f * a * c; U[7] = 2.f * c * d + 2.f * a * b; U[8] = a * a - b * b - c * c + d * d;
}
__device__ __forceinline__ f3 rot(const float* U, f3 r) {
    return {U[0] * r.x + U[1] * r.y + U[2] * r.z, U[3] * r.x + U[4] * r.y + U[5] * r.z,
            U[6] * r.x + U[7] * r.y + U[8] * r.z};
}

__device__ __forceinline__ bool acceptable_ids(int rule, int a, int b) {
    if (rule == 0) return (unsigned(a) >> 4) != (unsigned(b) >> 4);
    if (rule == 1) return (a - b > 1) || (b - a > 1);
    return (a - b > 2) || (b - a > 2);
}

// Threefry-4x32-20 (Salmon et al. 2011): the counter-based generator of the
// reference's random streams (src/random.h:19-67), key (seed, stream, 0, 0)
__device__ __forceinline__ uint32_t rotl32(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }
__device__ inline void threefry4x32(const uint32_t c[4], const uint32_t k[4], uint32_t out[4]) {
    const int R[8][2] = {{10, 26}, {11, 21}, {13, 27}, {23, 5}, {6, 20}, {17, 11}, {25, 10}, {18, 20}};
    uint32_t ks[5] = {k[0], k[1], k[2], k[3], 0x1BD11BDAu ^ k[0] ^ k[1] ^ k[2] ^ k[3]};
    uint32_t x[4];
    for (int i = 0; i < 4; ++i) x[i] = c[i] + ks[i];
#pragma unroll
    for (int r = 0; r < 20; ++r) {
        if (r % 2 == 0) {
            x[0] += x[1]; x[1] = rotl32(x[1], R[r % 8][0]); x[1] ^= x[0];
            x[2] += x[3]; x[3] = rotl32(x[3], R[r % 8][1]); x[3] ^= x[2];
        } else {
            x[0] += x[3]; x[3] = rotl32(x[3], R[r % 8][0]); x[3] ^= x[0];
            x[2] += x[1]; x[1] = rotl32(x[1], R[r % 8][1]); x[1] ^= x[2];
        }
        if (r % 4 == 3) {
            uint32_t s = uint32_t(r / 4 + 1);
            for (int i = 0; i < 4; ++i) x[i] += ks[(s + uint32_t(i)) % 5];
            x[3] += s;
        }
    }
    for (int i = 0; i < 4; ++i) out[i] = x[i];
}
// uniform in (0, 1] (r123::u01<float>) and a Box-Muller pair from two words
// (r123::boxmuller: angle from the signed word, radius from the unsigned one)
__device__ __forceinline__ float u01f(uint32_t b) { return float(b) * (1.f / 4294967296.f) + (0.5f / 4294967296.f); }
__device__ __forceinline__ void box_muller(uint32_t b0, uint32_t b1, float& x, float& y) {
    const float PIf = 3.1415926535897932f;
    float a = PIf * (float(int32_t(b0)) * (1.f / 2147483648.f) + (0.5f / 2147483648.f));
    float r = sqrtf(-2.f * logf(u01f(b1)));
    x = sinf(a) * r;
    y = cosf(a) * r;
}

__device__ __forceinline__ int grid_stride_start() { return blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ int grid_stride() { return gridDim.x * blockDim.x; }

}  // namespace ug
