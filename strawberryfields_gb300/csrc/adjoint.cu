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
// load feeds RR complex FMAs.  The loads of the CTA's next tile are issued
// before the contraction of the current one, so they are in flight while it
// runs.  Grid: about 8 CTAs per SM over all blocks, largest blocks first;
// kernels are compiled per cutoff bucket so registers match the block size.
// Partial C's of each CTA go to `cpart` ([gridDim.x][entries], FP64); a
// separate deterministic reduction sums them.
#include "apply.cuh"

template <int S> struct RRof { static const int value = (S + 3) / 4; };

// Loads of one column of lam_out and psi_in (S values each) into registers.
template <typename CT, int S>
__device__ __forceinline__ void adj_load(const CT* __restrict__ psi_in, const CT* __restrict__ lam_out,
                                         const AxisView& v, int D, const BlockGeom& g, int64_t j, CT* lam,
                                         CT* psi) {
  if (j < v.ncols) {
    const int64_t base = col_base(v, j, D) + g.boff;
#pragma unroll
    for (int u = 0; u < S; ++u) {
      lam[u] = __ldg(lam_out + base + u * g.step);
      psi[u] = __ldg(psi_in + base + u * g.step);
    }
  } else {
#pragma unroll
    for (int u = 0; u < S; ++u) {
      lam[u] = czero<CT>();
      psi[u] = czero<CT>();
    }
  }
}

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
  CT lam[S], psi[S];
  int64_t t = blockIdx.x;
  if (t < ntiles) adj_load<CT, S>(psi_in, lam_out, v, D, g, t * TILE + tid, lam, psi);
  for (; t < ntiles; t += gridDim.x) {
    const int64_t j = t * TILE + tid;
#pragma unroll
    for (int u = 0; u < S; ++u) {
      lam_s[u * LD + tid] = lam[u];
      psi_s[u * LD + tid] = psi[u];
    }
    if (write_lam && j < v.ncols) {
      const int64_t base = col_base(v, j, D) + g.boff;
#pragma unroll
      for (int w = 0; w < S; ++w) {
        CT a = czero<CT>();
#pragma unroll
        for (int u = 0; u < S; ++u) cfma(a, MsH[w * S + u], lam[u]);
        lam_in[base + w * g.step] = a;
      }
    }
    __syncthreads();
    // next tile's loads are in flight while this tile's contraction runs
    const int64_t tn = t + gridDim.x;
    if (tn < ntiles) adj_load<CT, S>(psi_in, lam_out, v, D, g, tn * TILE + tid, lam, psi);
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
  // large blocks (beyond the unrolled buckets): thread per C entry over this
  // CTA's share of the columns, then lam_in per column
  const int S = g.s;
  const int64_t per = (v.ncols + gridDim.x - 1) / gridDim.x;
  int64_t j0 = blockIdx.x * per, j1 = j0 + per;
  if (j1 > v.ncols) j1 = v.ncols;
  for (int e = threadIdx.x; e < S * S; e += blockDim.x) {
    int u = e / S, w = e - u * S;
    double2 a = make_double2(0.0, 0.0);
    for (int64_t j = j0; j < j1; ++j) {
      const int64_t base = col_base(v, j, D) + g.boff;
      double2 ld = to_d(lam_out[base + u * g.step]), pd = to_d(psi_in[base + w * g.step]);
      cfma_conj(a, ld, pd);
    }
    int aa = g.rev ? S - 1 - u : u, bb = g.rev ? S - 1 - w : w;
    cpart[(int64_t)blockIdx.x * nent + g.moff + aa * S + bb] = a;
  }
  if (!write_lam) return;
  for (int64_t j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    const int64_t base = col_base(v, j, D) + g.boff;
    for (int w = 0; w < S; ++w) {
      CT a = czero<CT>();
      for (int u = 0; u < S; ++u) cfma(a, MsH[w * S + u], lam_out[base + u * g.step]);
      lam_in[base + w * g.step] = a;
    }
  }
}

template <typename CT, int S, int DMAX, int TILE>
struct AdjDispatch {
  __device__ __forceinline__ static void run(const CT* psi_in, const CT* lam_out, CT* lam_in, const AxisView& v,
                                             int D, const CT* MsH, CT* lam_s, CT* psi_s, const BlockGeom& g,
                                             double2* cpart, int64_t nent, int write_lam) {
    if (g.s == S) adjoint_body<CT, S, TILE>(psi_in, lam_out, lam_in, v, D, MsH, lam_s, psi_s, g, cpart, nent, write_lam);
    else AdjDispatch<CT, S + 1, DMAX, TILE>::run(psi_in, lam_out, lam_in, v, D, MsH, lam_s, psi_s, g, cpart, nent, write_lam);
  }
};
template <typename CT, int DMAX, int TILE>
struct AdjDispatch<CT, DMAX + 1, DMAX, TILE> {
  __device__ __forceinline__ static void run(const CT* psi_in, const CT* lam_out, CT* lam_in, const AxisView& v,
                                             int D, const CT* MsH, CT*, CT*, const BlockGeom& g,
                                             double2* cpart, int64_t nent, int write_lam) {
    adjoint_generic<CT, TILE>(psi_in, lam_out, lam_in, v, D, MsH, g, cpart, nent, write_lam);
  }
};

template <typename CT, int TILE, int DMAX>
__global__ void __launch_bounds__(TILE) adjoint_block_kernel(const CT* __restrict__ psi_in,
                                                             const CT* __restrict__ lam_out,
                                                             CT* __restrict__ lam_in, AxisView v, int D,
                                                             int layout, const double2* __restrict__ mat,
                                                             int mflags, double2* __restrict__ cpart,
                                                             int64_t nent, int write_lam, BatchArg bt) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  psi_in += blockIdx.z * bt.state_stride;
  lam_out += blockIdx.z * bt.state_stride;
  if (write_lam) lam_in += blockIdx.z * bt.state_stride;
  mat += blockIdx.z * bt.mat_stride;
  cpart += blockIdx.z * bt.part_stride;
  const int b = layout == LAYOUT_DENSE ? 0 : block_of_y(D, blockIdx.y);
  const BlockGeom g = block_geom(v, D, layout, b, (mflags & MF_SWAP) ? 1 : 0);
  const int s = g.s;
  const int rows = 4 * ((s + 3) / 4);
  CT* MsH = reinterpret_cast<CT*>(smem_raw);
  CT* lam_s = MsH + s * s;
  CT* psi_s = lam_s + rows * (TILE + 1);
  if (write_lam) stage_block(MsH, mat, g, mflags | MF_ADJOINT);
  // zero the padding rows once (rows s..rows-1 stay zero)
  for (int e = threadIdx.x; e < (rows - s) * (TILE + 1); e += blockDim.x) {
    lam_s[s * (TILE + 1) + e] = czero<CT>();
    psi_s[s * (TILE + 1) + e] = czero<CT>();
  }
  __syncthreads();
  AdjDispatch<CT, 1, DMAX, TILE>::run(psi_in, lam_out, lam_in, v, D, MsH, lam_s, psi_s, g, cpart, nent, write_lam);
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
  // about 8 CTAs per SM in total: several waves, largest blocks scheduled first
  int target = (8 * fock_num_sms() + nblk - 1) / nblk;
  if (target < 1) target = 1;
  int64_t g = ntiles < target ? ntiles : target;
  return (int)(g < 1 ? 1 : g);
}

int64_t adjoint_scratch_entries(int dtype, const AxisView& v, int D, int layout) {
  return (int64_t)adjoint_grid_x(dtype, v, D, layout) * layout_entries(layout, D);
}

template <typename CT, int TILE, int DMAX>
static int launch_adj_t(const void* psi_in, const void* lam_out, void* lam_in, const AxisView& v, int D,
                        int layout, const double2* mat, int mflags, double2* cpart, int gx, size_t sm,
                        cudaStream_t st, const BatchArg& bt) {
  const int nblk = layout == LAYOUT_DENSE ? 1 : 2 * D - 1;
  if (bt.nb < 1 || bt.nb > 65535) return fock_set_error(FOCK_ERR_INVALID, "batch of %d circuits", bt.nb);
  const int64_t nent = layout_entries(layout, D);
  auto k = adjoint_block_kernel<CT, TILE, DMAX>;
  if (sm > 48 * 1024) FOCK_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  dim3 grid(gx, nblk, bt.nb);
  k<<<grid, TILE, sm, st>>>((const CT*)psi_in, (const CT*)lam_out, (CT*)lam_in, v, D, layout, mat, mflags, cpart,
                            nent, lam_in != nullptr, bt);
  FOCK_LAUNCH_CHECK("adjoint_block_kernel");
  return FOCK_OK;
}

template <typename CT, int TILE>
static int launch_adj_d(const void* psi_in, const void* lam_out, void* lam_in, const AxisView& v, int D,
                        int layout, const double2* mat, int mflags, double2* cpart, int gx, size_t sm,
                        cudaStream_t st, const BatchArg& bt) {
  switch (dmax_bucket(D)) {
    case 4: return launch_adj_t<CT, TILE, 4>(psi_in, lam_out, lam_in, v, D, layout, mat, mflags, cpart, gx, sm, st, bt);
    case 8: return launch_adj_t<CT, TILE, 8>(psi_in, lam_out, lam_in, v, D, layout, mat, mflags, cpart, gx, sm, st, bt);
    case 12: return launch_adj_t<CT, TILE, 12>(psi_in, lam_out, lam_in, v, D, layout, mat, mflags, cpart, gx, sm, st, bt);
    case 16: return launch_adj_t<CT, TILE, 16>(psi_in, lam_out, lam_in, v, D, layout, mat, mflags, cpart, gx, sm, st, bt);
    case 20: return launch_adj_t<CT, TILE, 20>(psi_in, lam_out, lam_in, v, D, layout, mat, mflags, cpart, gx, sm, st, bt);
    case 24: return launch_adj_t<CT, TILE, 24>(psi_in, lam_out, lam_in, v, D, layout, mat, mflags, cpart, gx, sm, st, bt);
    default: return launch_adj_t<CT, TILE, 0>(psi_in, lam_out, lam_in, v, D, layout, mat, mflags, cpart, gx, sm, st, bt);
  }
}

int launch_adjoint_partials(int dtype, const void* psi_in, const void* lam_out, void* lam_in,
                            const AxisView& v, int D, int layout, const double2* mat, int mflags,
                            double2* cpart, int gx, cudaStream_t st, const BatchArg& bt) {
  const size_t sm = adjoint_smem(dtype, D);
  if (dtype == FOCK_C64)
    return launch_adj_d<float2, 256>(psi_in, lam_out, lam_in, v, D, layout, mat, mflags, cpart, gx, sm, st, bt);
  return launch_adj_d<double2, 128>(psi_in, lam_out, lam_in, v, D, layout, mat, mflags, cpart, gx, sm, st, bt);
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

