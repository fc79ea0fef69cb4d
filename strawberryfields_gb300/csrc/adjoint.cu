// Adjoint (reverse-sweep) kernel: rows A1-A3 of the hot path.
//
// For one op psi_out = M psi_in (M dense D x D or photon-number blocks) and the
// incoming adjoint lam_out = dL/dpsi_out (torch convention dL/dRe + i dL/dIm):
//   lam_in  = M^dagger lam_out                          (per column)
//   C[u][v] = sum_columns conj(lam_out[u]) psi_in[v]     (per block)
// so that dL/dtheta = Re sum_{u,v} C[u][v] dM[u][v]/dtheta -- the quantity the
// reference's TF backend forms as Re sum dy * conj(dU) in its custom gradients
// (strawberryfields/backends/tfbackend/ops.py:190-204, 318-332, 349-366,
// 421-438).
//
// Tiling: a CTA stages TILE columns of lam_out and psi_in in shared memory
// (each thread loads one column, so global reads are coalesced across
// consecutive columns), computes its column of lam_in from registers, then
// the CTA forms the s x s outer-product sum C over the tile as a small
// register-tiled GEMM: 16 owners hold an RR x RR sub-block each (RR =
// ceil(s/4)), NG = TILE/16 groups split the tile's columns, so every shared
// load feeds RR complex FMAs.  Partial C's of each CTA go to `cpart`
// ([gridDim.x][entries], FP64); a separate deterministic reduction sums them.
#include "apply.cuh"

template <int S> struct RRof { static const int value = (S + 3) / 4; };

template <typename CT, int S, int TILE>
__device__ __forceinline__ void adjoint_body(const CT* __restrict__ psi_in, const CT* __restrict__ lam_out,
                                             CT* __restrict__ lam_in, const AxisView& v, int D,
                                             const CT* MsH, CT* lam_s, CT* psi_s, const BlockGeom& g,
                                             double2* __restrict__ cpart, int64_t nent, int write_lam) {
  constexpr int RR = RRof<S>::value;
  constexpr int NG = TILE / 16;
  constexpr int LD = TILE + 1;  // padded row stride (elements)
  const int tid = threadIdx.x;
  const int owner = tid / NG, grp = tid - owner * NG;
  const int ro = owner >> 2, co = owner & 3;
  CT acc[RR][RR];
#pragma unroll
  for (int r = 0; r < RR; ++r)
#pragma unroll
    for (int c = 0; c < RR; ++c) acc[r][c] = czero<CT>();

  const int64_t ntiles = (v.ncols + TILE - 1) / TILE;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t j = t * TILE + tid;
    if (j < v.ncols) {
      const int64_t base = col_base(v, j, D) + g.boff;
      CT lam[S];
#pragma unroll
      for (int u = 0; u < S; ++u) {
        lam[u] = __ldg(lam_out + base + u * g.step);
        lam_s[u * LD + tid] = lam[u];
        psi_s[u * LD + tid] = __ldg(psi_in + base + u * g.step);
      }
      if (write_lam) {
#pragma unroll
        for (int w = 0; w < S; ++w) {
          CT a = czero<CT>();
#pragma unroll
          for (int u = 0; u < S; ++u) cfma(a, MsH[w * S + u], lam[u]);
          lam_in[base + w * g.step] = a;
        }
      }
    } else {
#pragma unroll
      for (int u = 0; u < S; ++u) {
        lam_s[u * LD + tid] = czero<CT>();
        psi_s[u * LD + tid] = czero<CT>();
      }
    }
    __syncthreads();
#pragma unroll 4
    for (int step = 0; step < TILE / NG; ++step) {
      const int col = step * NG + grp;
      CT lv[RR], pv[RR];
#pragma unroll
      for (int r = 0; r < RR; ++r) lv[r] = lam_s[(ro * RR + r) * LD + col];
#pragma unroll
      for (int c = 0; c < RR; ++c) pv[c] = psi_s[(co * RR + c) * LD + col];
#pragma unroll
      for (int r = 0; r < RR; ++r)
#pragma unroll
        for (int c = 0; c < RR; ++c) cfma_conj(acc[r][c], lv[r], pv[c]);
    }
    __syncthreads();
  }
  // reduce over the NG groups of each owner (adjacent lanes)
#pragma unroll
  for (int off = NG / 2; off > 0; off >>= 1) {
#pragma unroll
    for (int r = 0; r < RR; ++r)
#pragma unroll
      for (int c = 0; c < RR; ++c) {
        acc[r][c].x += __shfl_xor_sync(0xffffffffu, acc[r][c].x, off);
        acc[r][c].y += __shfl_xor_sync(0xffffffffu, acc[r][c].y, off);
      }
  }
  if (grp == 0) {
    double2* dst = cpart + (int64_t)blockIdx.x * nent + g.moff;
#pragma unroll
    for (int r = 0; r < RR; ++r)
#pragma unroll
      for (int c = 0; c < RR; ++c) {
        int u = ro * RR + r, w = co * RR + c;
        if (u < S && w < S) {
          int a = g.rev ? S - 1 - u : u;
          int b = g.rev ? S - 1 - w : w;
          dst[a * S + b] = to_d(acc[r][c]);
        }
      }
  }
}

template <typename CT, int TILE>
__device__ void adjoint_generic(const CT* __restrict__ psi_in, const CT* __restrict__ lam_out,
                                CT* __restrict__ lam_in, const AxisView& v, int D, const CT* MsH,
                                const BlockGeom& g, double2* __restrict__ cpart, int64_t nent,
                                int write_lam) {
  // large blocks (s > 24): thread per C entry over all columns, then lam_in per column
  const int S = g.s;
  for (int e = threadIdx.x; e < S * S; e += blockDim.x) {
    int u = e / S, w = e - u * S;
    double2 a = make_double2(0.0, 0.0);
    const int64_t ntiles = (v.ncols + gridDim.x - 1) / gridDim.x;
    int64_t j0 = blockIdx.x * ntiles, j1 = j0 + ntiles;
    if (j1 > v.ncols) j1 = v.ncols;
    for (int64_t j = j0; j < j1; ++j) {
      const int64_t base = col_base(v, j, D) + g.boff;
      CT l = lam_out[base + u * g.step], p = psi_in[base + w * g.step];
      double2 ld = to_d(l), pd = to_d(p);
      cfma_conj(a, ld, pd);
    }
    int aa = g.rev ? S - 1 - u : u, bb = g.rev ? S - 1 - w : w;
    cpart[(int64_t)blockIdx.x * nent + g.moff + aa * S + bb] = a;
  }
  if (!write_lam) return;
  const int64_t per = (v.ncols + gridDim.x - 1) / gridDim.x;
  int64_t j0 = blockIdx.x * per, j1 = j0 + per;
  if (j1 > v.ncols) j1 = v.ncols;
  for (int64_t j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    const int64_t base = col_base(v, j, D) + g.boff;
    for (int w = 0; w < S; ++w) {
      CT a = czero<CT>();
      for (int u = 0; u < S; ++u) cfma(a, MsH[w * S + u], lam_out[base + u * g.step]);
      lam_in[base + w * g.step] = a;
    }
  }
}

#define ADJ_CASE(N) \
  case N: adjoint_body<CT, N, TILE>(psi_in, lam_out, lam_in, v, D, MsH, lam_s, psi_s, g, cpart, nent, write_lam); break;

template <typename CT, int TILE>
__global__ void __launch_bounds__(TILE) adjoint_block_kernel(const CT* __restrict__ psi_in,
                                                             const CT* __restrict__ lam_out,
                                                             CT* __restrict__ lam_in, AxisView v, int D,
                                                             int layout, const double2* __restrict__ mat,
                                                             int mflags, double2* __restrict__ cpart,
                                                             int64_t nent, int write_lam) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const BlockGeom g = block_geom(v, D, layout, blockIdx.y, (mflags & MF_SWAP) ? 1 : 0);
  const int s = g.s;
  const int rows = 4 * ((s + 3) / 4);
  CT* MsH = reinterpret_cast<CT*>(smem_raw);
  CT* lam_s = MsH + s * s;
  CT* psi_s = lam_s + rows * (TILE + 1);
  stage_block(MsH, mat, g, mflags | MF_ADJOINT);
  // zero the padding rows once (rows s..rows-1 stay zero)
  for (int e = threadIdx.x; e < (rows - s) * (TILE + 1); e += blockDim.x) {
    lam_s[s * (TILE + 1) + e] = czero<CT>();
    psi_s[s * (TILE + 1) + e] = czero<CT>();
  }
  __syncthreads();
  switch (s) {
    ADJ_CASE(1) ADJ_CASE(2) ADJ_CASE(3) ADJ_CASE(4) ADJ_CASE(5) ADJ_CASE(6)
    ADJ_CASE(7) ADJ_CASE(8) ADJ_CASE(9) ADJ_CASE(10) ADJ_CASE(11) ADJ_CASE(12)
    ADJ_CASE(13) ADJ_CASE(14) ADJ_CASE(15) ADJ_CASE(16) ADJ_CASE(17) ADJ_CASE(18)
    ADJ_CASE(19) ADJ_CASE(20) ADJ_CASE(21) ADJ_CASE(22) ADJ_CASE(23) ADJ_CASE(24)
    default: adjoint_generic<CT, TILE>(psi_in, lam_out, lam_in, v, D, MsH, g, cpart, nent, write_lam); break;
  }
}

static int tile_of(int dtype) { return dtype == FOCK_C64 ? 256 : 128; }

static size_t adjoint_smem(int dtype, int D) {
  const int esz = dtype == FOCK_C64 ? 8 : 16;
  const int rows = 4 * ((D + 3) / 4);
  return (size_t)esz * ((size_t)D * D + 2 * (size_t)rows * (tile_of(dtype) + 1));
}

int adjoint_grid_x(int dtype, const AxisView& v, int D, int layout) {
  const int nblk = layout == LAYOUT_DENSE ? 1 : 2 * D - 1;
  const int64_t ntiles = (v.ncols + tile_of(dtype) - 1) / tile_of(dtype);
  int target = (2 * fock_num_sms() + nblk - 1) / nblk;
  if (target < 1) target = 1;
  int64_t g = ntiles < target ? ntiles : target;
  return (int)(g < 1 ? 1 : g);
}

int64_t adjoint_scratch_entries(int dtype, const AxisView& v, int D, int layout) {
  return (int64_t)adjoint_grid_x(dtype, v, D, layout) * layout_entries(layout, D);
}

int launch_adjoint_partials(int dtype, const void* psi_in, const void* lam_out, void* lam_in,
                            const AxisView& v, int D, int layout, const double2* mat, int mflags,
                            double2* cpart, int gx, cudaStream_t st) {
  const int nblk = layout == LAYOUT_DENSE ? 1 : 2 * D - 1;
  const int64_t nent = layout_entries(layout, D);
  dim3 grid(gx, nblk);
  const size_t sm = adjoint_smem(dtype, D);
  const int write_lam = lam_in != nullptr;
  if (dtype == FOCK_C64) {
    auto k = adjoint_block_kernel<float2, 256>;
    if (sm > 48 * 1024) FOCK_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k<<<grid, 256, sm, st>>>((const float2*)psi_in, (const float2*)lam_out, (float2*)lam_in, v, D, layout, mat,
                             mflags, cpart, nent, write_lam);
  } else {
    auto k = adjoint_block_kernel<double2, 128>;
    if (sm > 48 * 1024) FOCK_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k<<<grid, 128, sm, st>>>((const double2*)psi_in, (const double2*)lam_out, (double2*)lam_in, v, D, layout,
                             mat, mflags, cpart, nent, write_lam);
  }
  FOCK_LAUNCH_CHECK("adjoint_block_kernel");
  return FOCK_OK;
}

// cout[e] = sum_x cpart[x][e]  (one warp per entry, fixed summation order)
__global__ void reduce_partials_kernel(const double2* __restrict__ cpart, int gx, int64_t nent,
                                       double2* __restrict__ cout) {
  const int lane = threadIdx.x & 31;
  const int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (e >= nent) return;
  double2 a = make_double2(0.0, 0.0);
  for (int x = lane; x < gx; x += 32) {
    double2 p = cpart[(int64_t)x * nent + e];
    a.x += p.x;
    a.y += p.y;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    a.x += __shfl_xor_sync(0xffffffffu, a.x, off);
    a.y += __shfl_xor_sync(0xffffffffu, a.y, off);
  }
  if (lane == 0) cout[e] = a;
}

int launch_reduce_partials(const double2* cpart, int gx, int64_t nent, double2* cout, cudaStream_t st) {
  const int64_t threads = nent * 32;
  const int64_t blocks = (threads + 255) / 256;
  reduce_partials_kernel<<<(unsigned)blocks, 256, 0, st>>>(cpart, gx, nent, cout);
  FOCK_LAUNCH_CHECK("reduce_partials_kernel");
  return FOCK_OK;
}

