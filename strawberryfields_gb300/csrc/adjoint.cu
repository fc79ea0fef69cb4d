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
// load feeds RR complex FMAs.  Tiles arrive in shared memory through
// cp.async (no register staging), which keeps registers low enough for three
// resident CTAs per SM.  Grid: about 8 CTAs per SM over all blocks, largest
// blocks first; kernels are compiled per cutoff bucket.
// Partial C's of each CTA go to `cpart` ([gridDim.x][entries], FP64); a
// separate deterministic reduction sums them.
#include "block_body.cuh"

#include <string.h>

#include <algorithm>

template <typename CT, int TILE, int DMAX>
__global__ void __launch_bounds__(TILE, AdjMinBlocks<CT, DMAX>::value)
    adjoint_block_kernel(const CT* __restrict__ psi_in, const CT* __restrict__ lam_out, CT* __restrict__ lam_in,
                         AxisView v, int D, int layout, const double2* __restrict__ mat, int mflags,
                         double2* __restrict__ cpart, AdjSched sc, int write_lam, BatchArg bt) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // which block this CTA serves, and its rank x among that block's CTAs
  int y = 0, xrank;
  if (sc.interleave) {
    y = (int)blockIdx.x % sc.nblk;
    xrank = (int)blockIdx.x / sc.nblk;
  } else {
    while (y + 1 < sc.nblk && (int)blockIdx.x >= sc.start[y + 1]) ++y;
    xrank = (int)blockIdx.x - sc.start[y];
  }
  const int gxb = sc.gx[y];
  psi_in += blockIdx.z * bt.state_stride;
  lam_out += blockIdx.z * bt.state_stride;
  if (write_lam) lam_in += blockIdx.z * bt.state_stride;
  mat = mat_batch(mat, blockIdx.z * bt.mat_stride, mflags);
  cpart += blockIdx.z * bt.part_stride;
  const int b = layout == LAYOUT_DENSE ? 0 : block_of_y(D, y);
  const BlockGeom g = block_geom(v, D, layout, b, (mflags & MF_SWAP) ? 1 : 0);
  const int s = g.s;
  const int rows = 4 * ((s + 3) / 4);
  // partial slot of this CTA (stored-orientation block)
  const int bs = layout == LAYOUT_DENSE ? 0 : ((layout == LAYOUT_DIFF && (mflags & MF_SWAP)) ? 2 * D - 2 - b : b);
  double2* mypart = cpart + sc.part_off[bs] + (int64_t)xrank * s * s;
  CT* MsH = reinterpret_cast<CT*>(smem_raw);
  CT* lam_s = MsH + ((ms_slots(sizeof(CT) == 8 ? FOCK_C64 : FOCK_C128, D) + 1) & ~(size_t)1);
  CT* psi_s = lam_s + rows * (TILE + 1);
  // the matrix was built before the sweep: stage it while the previous op
  // finishes
  if (write_lam) StageDispatch<CT, kSStep, DMAX>::run(MsH, mat, g, mflags | MF_ADJOINT);
  pdl_wait();
  pdl_launch_dependents();
  AdjDispatch<CT, kSStep, DMAX, TILE>::run(psi_in, lam_out, lam_in, v, D, MsH, mat, mflags, lam_s, psi_s, g, mypart,
                                      xrank, gxb, write_lam, 1);
}

static int tile_of(int dtype) { return dtype == FOCK_C64 ? 256 : 128; }

static size_t adjoint_smem(int dtype, int D) {
  const int esz = dtype == FOCK_C64 ? 8 : 16;
  const size_t ms = (ms_slots(dtype, D) + 1) & ~(size_t)1;
  // cutoffs past the unrolled buckets run adjoint_generic, which stages only
  // the matrix (the lam / psi tiles of the unrolled body would not fit shared
  // memory there: about 300 KB at cutoff 60)
  if (dmax_bucket(D) == 0) return (size_t)esz * ms;
  const int rows = 4 * ((D + 3) / 4);
  // matrix + the lam and psi tiles
  return (size_t)esz * (ms + 2 * (size_t)rows * (tile_of(dtype) + 1));
}

AdjSched make_adj_sched(int dtype, const AxisView& v, int D, int layout, int nb, int ctas_per_sm) {
  AdjSched sc;
  memset(&sc, 0, sizeof(sc));
  sc.nblk = layout == LAYOUT_DENSE ? 1 : 2 * D - 1;
  if (sc.nblk > ADJ_MAX_BLOCKS) sc.nblk = 0;  // cutoff beyond FOCK_MAX_CUTOFF: callers reject it first
  const int64_t ntiles = (v.ncols + tile_of(dtype) - 1) / tile_of(dtype);
  // the same number of CTAs for every block (small blocks are memory-bound
  // and need as many as large ones), ctas_per_sm CTAs per SM over all nb
  // circuits of a batch (grid.z); largest blocks come first in the flat grid
  // so they start first
  const int target = std::max(1, std::max(ctas_per_sm, 1) * fock_num_sms() / std::max(nb, 1));
  // innermost-pair ops: one column tile per CTA, so the CTAs of all blocks
  // that read a tile's planes run together (a CTA that walks many tiles
  // drifts away from the other blocks' CTAs, and the planes come from DRAM
  // again) -- as far as 64 MB of partial sums per launch allow
  int64_t per_block = (target + sc.nblk - 1) / sc.nblk;
  if (interleave_blocks(layout, v)) {
    const int64_t per_tile = (layout == LAYOUT_DENSE ? (int64_t)D * D : blk_total(D)) * (int64_t)sizeof(double2) *
                             std::max(nb, 1);
    per_block = std::max<int64_t>(per_block, std::min<int64_t>(ntiles, (64ll << 20) / per_tile));
  }
  int64_t part = 0;
  int start = 0;
  for (int y = 0; y < sc.nblk; ++y) {
    int64_t g = per_block;
    if (g < 1) g = 1;
    if (g > ntiles) g = ntiles;
    sc.gx[y] = (int)g;
    sc.start[y] = start;
    start += (int)g;
  }
  sc.start[sc.nblk] = start;
  sc.total = start;
  // every block has the same CTA count, so the interleaved order is a
  // permutation of the same grid
  sc.interleave = interleave_blocks(layout, v);
  // partial offsets by stored block index (gx depends only on the block size,
  // so a block and its mirror image have the same count)
  for (int bs = 0; bs < sc.nblk; ++bs) {
    const int s = layout == LAYOUT_DENSE ? D : blk_size(D, bs);
    // gx of a view block of the same size
    int g = 1;
    for (int y = 0; y < sc.nblk; ++y)
      if ((layout == LAYOUT_DENSE ? D : blk_size(D, block_of_y(D, y))) == s) { g = sc.gx[y]; break; }
    sc.part_off[bs] = part;
    part += (int64_t)g * s * s;
  }
  sc.part_entries = part;
  return sc;
}

__global__ void reduce_sched_kernel(const double2* __restrict__ cpart, AdjSched sc, int D, int layout,
                                    double2* __restrict__ cout, int64_t part_stride, int64_t out_stride) {
  pdl_wait();
  pdl_launch_dependents();
  const int lane = threadIdx.x & 31;
  const int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  cpart += blockIdx.y * part_stride;
  cout += blockIdx.y * out_stride;
  const int64_t nent = layout == LAYOUT_DENSE ? (int64_t)D * D : blk_total(D);
  if (e >= nent) return;
  // stored block of entry e
  int bs = 0;
  int64_t off = 0;
  int s = D;
  if (layout != LAYOUT_DENSE) {
    for (bs = 0; bs < 2 * D - 1; ++bs) {
      s = blk_size(D, bs);
      if (e < off + (int64_t)s * s) break;
      off += (int64_t)s * s;
    }
  }
  int g = 1;
  for (int y = 0; y < sc.nblk; ++y)
    if ((layout == LAYOUT_DENSE ? D : blk_size(D, block_of_y(D, y))) == s) { g = sc.gx[y]; break; }
  const int64_t le = e - off;
  double2 a = make_double2(0.0, 0.0);
  for (int x = lane; x < g; x += 32) {
    double2 p = cpart[sc.part_off[bs] + (int64_t)x * s * s + le];
    a.x += p.x;
    a.y += p.y;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a.x += __shfl_xor_sync(0xffffffffu, a.x, o);
    a.y += __shfl_xor_sync(0xffffffffu, a.y, o);
  }
  if (lane == 0) cout[e] = a;
}

int launch_reduce_sched(const double2* cpart, const AdjSched& sc, int D, int layout, double2* cout, cudaStream_t st,
                        int nb, int64_t part_stride, int64_t out_stride, int pdl) {
  const int64_t nent = layout == LAYOUT_DENSE ? (int64_t)D * D : blk_total(D);
  const int64_t blocks = (nent * 32 + 255) / 256;
  FOCK_CUDA_TRY(launch_kernel(reduce_sched_kernel, dim3((unsigned)blocks, nb), dim3(256), 0, st, pdl, cpart, sc, D,
                               layout, cout, part_stride, out_stride));
  return FOCK_OK;
}

template <typename CT, int TILE, int DMAX>
static int launch_adj_t(const void* psi_in, const void* lam_out, void* lam_in, const AxisView& v, int D,
                        int layout, const double2* mat, int mflags, double2* cpart, const AdjSched& sc, size_t sm,
                        cudaStream_t st, const BatchArg& bt) {
  if (bt.nb < 1 || bt.nb > 65535) return fock_set_error(FOCK_ERR_INVALID, "batch of %d circuits", bt.nb);
  auto k = adjoint_block_kernel<CT, TILE, DMAX>;
  if (sm > 48 * 1024) FOCK_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  dim3 grid(sc.total, 1, bt.nb);
  FOCK_CUDA_TRY(launch_kernel(k, grid, dim3(TILE), sm, st, bt.pdl, (const CT*)psi_in, (const CT*)lam_out, (CT*)lam_in,
                               v, D, layout, mat, mflags, cpart, sc, (int)(lam_in != nullptr), bt));
  return FOCK_OK;
}

template <typename CT, int TILE>
static int launch_adj_d(const void* psi_in, const void* lam_out, void* lam_in, const AxisView& v, int D,
                        int layout, const double2* mat, int mflags, double2* cpart, const AdjSched& sc, size_t sm,
                        cudaStream_t st, const BatchArg& bt) {
  switch (dmax_bucket(D)) {
    case 4: return launch_adj_t<CT, TILE, 4>(psi_in, lam_out, lam_in, v, D, layout, mat, mflags, cpart, sc, sm, st, bt);
    case 8: return launch_adj_t<CT, TILE, 8>(psi_in, lam_out, lam_in, v, D, layout, mat, mflags, cpart, sc, sm, st, bt);
    case 12: return launch_adj_t<CT, TILE, 12>(psi_in, lam_out, lam_in, v, D, layout, mat, mflags, cpart, sc, sm, st, bt);
    case 16: return launch_adj_t<CT, TILE, 16>(psi_in, lam_out, lam_in, v, D, layout, mat, mflags, cpart, sc, sm, st, bt);
    case 20: return launch_adj_t<CT, TILE, 20>(psi_in, lam_out, lam_in, v, D, layout, mat, mflags, cpart, sc, sm, st, bt);
    case 24: return launch_adj_t<CT, TILE, 24>(psi_in, lam_out, lam_in, v, D, layout, mat, mflags, cpart, sc, sm, st, bt);
    default: return launch_adj_t<CT, TILE, 0>(psi_in, lam_out, lam_in, v, D, layout, mat, mflags, cpart, sc, sm, st, bt);
  }
}

int launch_adjoint_partials(int dtype, const void* psi_in, const void* lam_out, void* lam_in,
                            const AxisView& v, int D, int layout, const double2* mat, int mflags,
                            double2* cpart, const AdjSched& sc, cudaStream_t st, const BatchArg& bt) {
  const size_t sm = adjoint_smem(dtype, D);
  if (dtype == FOCK_C64)
    return launch_adj_d<float2, 256>(psi_in, lam_out, lam_in, v, D, layout, mat, mflags, cpart, sc, sm, st, bt);
  return launch_adj_d<double2, 128>(psi_in, lam_out, lam_in, v, D, layout, mat, mflags, cpart, sc, sm, st, bt);
}

// cout[e] = sum_x cpart[x][e]  (one warp per entry, fixed summation order)
__global__ void reduce_partials_kernel(const double2* __restrict__ cpart, int gx, int64_t nent,
                                       double2* __restrict__ cout, int64_t part_stride, int64_t out_stride) {
  pdl_wait();
  pdl_launch_dependents();
  const int lane = threadIdx.x & 31;
  // blockIdx.y: circuit of a batch
  cpart += blockIdx.y * part_stride;
  cout += blockIdx.y * out_stride;
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

int launch_reduce_partials(const double2* cpart, int gx, int64_t nent, double2* cout, cudaStream_t st, int nb,
                           int64_t part_stride, int64_t out_stride, int pdl) {
  const int64_t threads = nent * 32;
  const int64_t blocks = (threads + 255) / 256;
  FOCK_CUDA_TRY(launch_kernel(reduce_partials_kernel, dim3((unsigned)blocks, nb), dim3(256), 0, st, pdl, cpart, gx, nent,
                               cout, part_stride, out_stride));
  return FOCK_OK;
}


// every op's partial sums at once.  One CTA per chunk of ec consecutive C
// entries of one op (ec = 32, 16 or 8 by the op's partial-row count gx): the
// CTA's K = 256 / ec row segments each sum rows x = k, k + K, ... of the
// chunk's entries (a row's entries are contiguous, so the loads are whole
// 128-byte lines or more), then the K segment sums of each entry are added
// in order.  The order is fixed by the plan, so the result does not depend on
// timing.
__global__ void __launch_bounds__(RED_THREADS)
    reduce_ops_kernel(const RedOp* __restrict__ ops, int n_ops, int D, const double2* __restrict__ cpart,
                      double2* __restrict__ carena, int64_t part_stride, int64_t out_stride) {
  pdl_wait();
  pdl_launch_dependents();
  __shared__ double2 red[RED_THREADS];
  cpart += blockIdx.y * part_stride;
  carena += blockIdx.y * out_stride;
  const int chunk = (int)blockIdx.x;
  int lo = 0, hi = n_ops - 1;
  while (lo < hi) {  // last op whose first chunk is <= this one
    const int mid = (lo + hi + 1) >> 1;
    if (ops[mid].chunk0 <= chunk) lo = mid;
    else hi = mid - 1;
  }
  const RedOp R = ops[lo];
  const int ec = R.ec, K = RED_THREADS / ec;
  const int i = threadIdx.x % ec, k = threadIdx.x / ec;
  const int64_t le = (int64_t)(chunk - R.chunk0) * ec + i;
  double2 a = make_double2(0.0, 0.0);
  if (le < R.nent) {
    // partial rows of entry le: [gx][nent] (plane), [gx][D*D] (dense), or
    // the entry's block [gx][s*s] at gx * (entries of the earlier blocks)
    const double2* src;
    int64_t stride;
    if (R.plane) {
      src = cpart + R.cpart_off + le;
      stride = R.nent;
    } else if (R.layout == LAYOUT_DENSE) {
      src = cpart + R.cpart_off + le;
      stride = (int64_t)D * D;
    } else {
      int bs = 0, s = 1;
      int64_t off = 0;
      for (bs = 0; bs < 2 * D - 1; ++bs) {
        s = blk_size(D, bs);
        if (le < off + (int64_t)s * s) break;
        off += (int64_t)s * s;
      }
      src = cpart + R.cpart_off + (int64_t)R.gx * off + (le - off);
      stride = (int64_t)s * s;
    }
    int x = k;
    for (; x + 3 * K < R.gx; x += 4 * K) {
      const double2 p0 = src[(int64_t)x * stride];
      const double2 p1 = src[(int64_t)(x + K) * stride];
      const double2 p2 = src[(int64_t)(x + 2 * K) * stride];
      const double2 p3 = src[(int64_t)(x + 3 * K) * stride];
      a.x += p0.x; a.y += p0.y;
      a.x += p1.x; a.y += p1.y;
      a.x += p2.x; a.y += p2.y;
      a.x += p3.x; a.y += p3.y;
    }
    for (; x < R.gx; x += K) {
      const double2 p = src[(int64_t)x * stride];
      a.x += p.x; a.y += p.y;
    }
  }
  red[threadIdx.x] = a;
  __syncthreads();
  if (k == 0 && le < R.nent) {
    for (int q = 1; q < K; ++q) {
      a.x += red[q * ec + i].x;
      a.y += red[q * ec + i].y;
    }
    carena[R.c_off + le] = a;
  }
}

int launch_reduce_ops(const RedOp* ops, int n_ops, int64_t chunks, int D, const double2* cpart, double2* carena,
                      cudaStream_t st, int nb, int64_t part_stride, int64_t out_stride) {
  if (chunks <= 0) return FOCK_OK;
  if (chunks > 0x7fffffffLL) return fock_set_error(FOCK_ERR_INVALID, "too many reduction chunks");
  FOCK_CUDA_TRY(launch_kernel(reduce_ops_kernel, dim3((unsigned)chunks, nb), dim3(RED_THREADS), 0, st, 0,
                               ops, n_ops, D, cpart, carena, part_stride, out_stride));
  return FOCK_OK;
}
