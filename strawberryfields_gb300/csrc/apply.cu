// Gate application kernels (rows K1-K5 of the hot path).
//
// One kernel covers every non-diagonal op: a gate matrix stored as one dense
// D x D block (single-mode gates) or as 2D-1 photon-number blocks (beamsplitter
// / MZ conserve n1+n2, two-mode squeezing and the loss superoperator conserve
// n1-n2 -- the selection rules the reference exploits in
// fockbackend/circuit.py:307-365).  Grid: x over columns (one thread per
// column), y over blocks.  Each thread loads the s values of its block into
// registers (coalesced across the warp: consecutive threads take consecutive
// columns, i.e. consecutive addresses along the innermost non-gate axis),
// multiplies by the s x s block held in shared memory (broadcast reads) and
// stores s outputs.  The block size s is a compile-time constant through a
// switch, so the loads and the complex FMAs are fully unrolled.
#include "apply.cuh"

AxisView make_view1(int naxes, int D, int ax) {
  AxisView v;
  int64_t C = 1;
  for (int k = ax + 1; k < naxes; ++k) C *= D;
  int64_t A = 1;
  for (int k = 0; k < ax; ++k) A *= D;
  v.A = A; v.B = 1; v.C = C; v.s1 = C; v.s2 = 0;
  v.ncols = A * C;
  return v;
}

AxisView make_view2(int naxes, int D, int ax1, int ax2) {
  AxisView v;
  int64_t C = 1, B = 1, A = 1;
  for (int k = ax2 + 1; k < naxes; ++k) C *= D;
  for (int k = ax1 + 1; k < ax2; ++k) B *= D;
  for (int k = 0; k < ax1; ++k) A *= D;
  v.A = A; v.B = B; v.C = C;
  v.s2 = C;
  v.s1 = B * D * C;
  v.ncols = A * B * C;
  return v;
}

template <typename CT, int S>
__device__ __forceinline__ void apply_cols(const CT* __restrict__ in, CT* __restrict__ out,
                                           const AxisView& v, int D, const CT* Ms,
                                           const BlockGeom& g, int64_t j) {
  const int64_t base = col_base(v, j, D) + g.boff;
  const CT* p = in + base;
  CT x[S];
#pragma unroll
  for (int u = 0; u < S; ++u) x[u] = __ldg(p + u * g.step);
  CT* q = out + base;
#pragma unroll
  for (int w = 0; w < S; ++w) {
    CT acc = czero<CT>();
#pragma unroll
    for (int u = 0; u < S; ++u) cfma(acc, Ms[w * S + u], x[u]);
    q[w * g.step] = acc;
  }
}

template <typename CT>
__device__ void apply_cols_generic(const CT* __restrict__ in, CT* __restrict__ out, const AxisView& v,
                                   int D, const CT* Ms, const BlockGeom& g, int64_t j) {
  const int64_t base = col_base(v, j, D) + g.boff;
  const int S = g.s;
  for (int w = 0; w < S; ++w) {
    CT acc = czero<CT>();
    for (int u = 0; u < S; ++u) cfma(acc, Ms[w * S + u], in[base + u * g.step]);
    out[base + w * g.step] = acc;
  }
}

#define APPLY_CASE(N) case N: apply_cols<CT, N>(in, out, v, D, Ms, g, j); break;

template <typename CT>
__global__ void __launch_bounds__(256) apply_block_kernel(const CT* __restrict__ in, CT* __restrict__ out,
                                                          AxisView v, int D, int layout,
                                                          const double2* __restrict__ mat, int mflags) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CT* Ms = reinterpret_cast<CT*>(smem_raw);
  const BlockGeom g = block_geom(v, D, layout, blockIdx.y, (mflags & MF_SWAP) ? 1 : 0);
  stage_block(Ms, mat, g, mflags);
  __syncthreads();
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= v.ncols) return;
  switch (g.s) {
    APPLY_CASE(1) APPLY_CASE(2) APPLY_CASE(3) APPLY_CASE(4) APPLY_CASE(5) APPLY_CASE(6)
    APPLY_CASE(7) APPLY_CASE(8) APPLY_CASE(9) APPLY_CASE(10) APPLY_CASE(11) APPLY_CASE(12)
    APPLY_CASE(13) APPLY_CASE(14) APPLY_CASE(15) APPLY_CASE(16) APPLY_CASE(17) APPLY_CASE(18)
    APPLY_CASE(19) APPLY_CASE(20) APPLY_CASE(21) APPLY_CASE(22) APPLY_CASE(23) APPLY_CASE(24)
    default: apply_cols_generic<CT>(in, out, v, D, Ms, g, j); break;
  }
}

int launch_apply(int dtype, const void* in, void* out, const AxisView& v, int D, int layout,
                 const double2* mat, int mflags, cudaStream_t st) {
  if (v.ncols <= 0) return FOCK_OK;
  const int nblk = layout == LAYOUT_DENSE ? 1 : 2 * D - 1;
  const int64_t gx = (v.ncols + 255) / 256;
  if (gx > 0x7fffffffLL) return fock_set_error(FOCK_ERR_INVALID, "state too large");
  dim3 grid((unsigned)gx, nblk);
  if (dtype == FOCK_C64) {
    size_t sm = (size_t)D * D * sizeof(float2);
    if (sm > 48 * 1024)
      FOCK_CUDA_TRY(cudaFuncSetAttribute(apply_block_kernel<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    apply_block_kernel<float2><<<grid, 256, sm, st>>>((const float2*)in, (float2*)out, v, D, layout, mat, mflags);
  } else {
    size_t sm = (size_t)D * D * sizeof(double2);
    if (sm > 48 * 1024)
      FOCK_CUDA_TRY(cudaFuncSetAttribute(apply_block_kernel<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    apply_block_kernel<double2><<<grid, 256, sm, st>>>((const double2*)in, (double2*)out, v, D, layout, mat, mflags);
  }
  FOCK_LAUNCH_CHECK("apply_block_kernel");
  return FOCK_OK;
}
