// Shared device/host helpers for the GB300 Fock-basis simulator.
//
// State layout in HBM: a pure n-mode state is a C-order tensor [D]^n (mode 0
// slowest), a mixed state is [D]^(2n) with interleaved (ket, bra) axes per
// mode -- the layout of strawberryfields/backends/fockbackend/backend.py:50-56.
// Elements are interleaved complex pairs: float2 (complex64) or double2
// (complex128).  Gate matrices are always built and stored in FP64 (double2)
// and converted to the state precision when staged into shared memory.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include "../../include/fock_gb300.h"

#define FOCK_MAX_CUTOFF 64      // largest cutoff any kernel accepts
#define FOCK_MAX_TEMPLATE_D 24  // largest block size with a register-resident kernel
#define FOCK_MAX_AXES 64        // mixed states: 2 axes per mode

// ---------------------------------------------------------------------------
// complex arithmetic on float2 / double2
// ---------------------------------------------------------------------------
template <typename R> struct cplx;
template <> struct cplx<float> { typedef float2 T; };
template <> struct cplx<double> { typedef double2 T; };

__host__ __device__ __forceinline__ float2 mk(float a, float b) { return make_float2(a, b); }
__host__ __device__ __forceinline__ double2 mk(double a, double b) { return make_double2(a, b); }

template <typename C> __host__ __device__ __forceinline__ C czero();
template <> __host__ __device__ __forceinline__ float2 czero<float2>() { return make_float2(0.f, 0.f); }
template <> __host__ __device__ __forceinline__ double2 czero<double2>() { return make_double2(0.0, 0.0); }

template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) { a.x += b.x; a.y += b.y; return a; }
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b) {
  C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
template <typename C> __host__ __device__ __forceinline__ C cconj(C a) { a.y = -a.y; return a; }
// acc += a * b
template <typename C> __host__ __device__ __forceinline__ void cfma(C& acc, C a, C b) {
  acc.x = fma(a.x, b.x, acc.x); acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y); acc.y = fma(a.y, b.x, acc.y);
}
// acc += conj(a) * b
template <typename C> __host__ __device__ __forceinline__ void cfma_conj(C& acc, C a, C b) {
  acc.x = fma(a.x, b.x, acc.x); acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y); acc.y = fma(-a.y, b.x, acc.y);
}
template <typename C, typename S> __host__ __device__ __forceinline__ C cscale(C a, S s) { a.x *= s; a.y *= s; return a; }

// Packed FP32 pairs for the Blackwell paired FMA (fma.rn.f32x2: one
// instruction, two lanes, each rounded like a scalar fma).  A pair lives in a
// 64-bit register (low lane first), so a complex64 entry loaded from memory
// is already a pair.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float lo, float hi) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ float2 upk2(f32x2 v) {
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
  return r;
}
// a * b + c, lane by lane
__device__ __forceinline__ f32x2 ffma2(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

__device__ __forceinline__ float2 to_c(double2 v, float2*) { return make_float2((float)v.x, (float)v.y); }
__device__ __forceinline__ double2 to_c(double2 v, double2*) { return v; }
__device__ __forceinline__ double2 to_d(float2 v) { return make_double2(v.x, v.y); }
__device__ __forceinline__ double2 to_d(double2 v) { return v; }

// ---------------------------------------------------------------------------
// error reporting (host)
// ---------------------------------------------------------------------------
int fock_set_error(int code, const char* fmt, ...);
int fock_check_cuda(cudaError_t e, const char* what);

#define FOCK_CUDA_TRY(expr)                                  \
  do {                                                       \
    cudaError_t _e = (expr);                                 \
    if (_e != cudaSuccess) return fock_check_cuda(_e, #expr); \
  } while (0)

#define FOCK_LAUNCH_CHECK(what)                                       \
  do {                                                                \
    cudaError_t _e = cudaGetLastError();                              \
    if (_e != cudaSuccess) return fock_check_cuda(_e, what);          \
  } while (0)

// ---------------------------------------------------------------------------
// block-structured two-axis gates
// ---------------------------------------------------------------------------
// A beamsplitter-like gate conserves n1+n2 (kind SUM); a two-mode squeezer or
// the loss superoperator conserves n1-n2 (kind DIFF).  Each gate is stored as
// 2D-1 dense blocks, block b of size s_b = D - |b - (D-1)|, in block-major
// order [b][u][v] (u: output position, v: input position).
//   SUM : block b = N (total photons); position u <-> (k_lo+u, N-k_lo-u),
//         k_lo = max(0, N-(D-1)).
//   DIFF: block b = Delta + D - 1 (Delta = n1 - n2); position u <->
//         (m_lo+u, m_lo+u-Delta), m_lo = max(0, Delta).
// Total entries: D (2 D^2 + 1) / 3.
__host__ __device__ __forceinline__ int blk_size(int D, int b) {
  int d = b - (D - 1);
  return D - (d < 0 ? -d : d);
}
__host__ __device__ __forceinline__ int blk_offset(int D, int b) {
  // sum_{b' < b} s_{b'}^2
  int off = 0;
  if (b <= D) {
    // s = 1..b
    off = b * (b + 1) * (2 * b + 1) / 6;
  } else {
    off = D * (D + 1) * (2 * D + 1) / 6;  // blocks 0..D-1 (sizes 1..D)
    int k = b - D;                        // blocks D..b-1 with sizes D-1 .. D-k
    // sum_{s=D-k}^{D-1} s^2
    int hi = D - 1, lo = D - k;
    off += hi * (hi + 1) * (2 * hi + 1) / 6 - (lo - 1) * lo * (2 * lo - 1) / 6;
  }
  return off;
}
__host__ __device__ __forceinline__ int blk_total(int D) { return D * (2 * D * D + 1) / 3; }
// first coordinate (axis-1 index) of position 0 of block b
__host__ __device__ __forceinline__ int blk_lo(int D, int kind_sum, int b) {
  if (kind_sum) { int lo = b - (D - 1); return lo > 0 ? lo : 0; }
  int delta = b - (D - 1);
  return delta > 0 ? delta : 0;
}
// (i, j) coordinates of position u in block b
__host__ __device__ __forceinline__ void blk_coord(int D, int kind_sum, int b, int u, int& i, int& j) {
  int lo = blk_lo(D, kind_sum, b);
  i = lo + u;
  if (kind_sum) j = b - i;               // N - i
  else j = i - (b - (D - 1));            // i - Delta
}

// host-side launch helpers
int fock_num_sms();
