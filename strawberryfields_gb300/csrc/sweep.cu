// Persistent sweep kernels: a whole forward or adjoint sweep in one launch.
//
// For a small state (the 6-mode cutoff-12 CV-QNN ket is 24 MB and stays in
// L2) one op moves a few microseconds' worth of bytes, while a kernel launch
// costs its ramp-up, its last partial wave and its drain on top.  Here one
// cooperative launch keeps every CTA resident for the whole sweep and walks
// the plan's ops in order; between two ops all CTAs meet at a grid barrier
// (release/acquire through an arrival counter and a generation word), so op
// k+1 reads what op k wrote.  Each op's work is the block kernels' work
// (block_body.cuh): forward items are (block, 256-column tile) pairs dealt
// round-robin to the CTAs; the adjoint uses a per-op CTA schedule whose
// partial C sums go to a per-op region that the same launch reduces, in a
// fixed order, after the last op.
//
// Every spin has an iteration limit (SweepSync::spin_limit polls, 2^24 by
// default, about a second): a barrier that does not complete sets the error
// flag and the kernel returns (the host reads the flag with
// fock_plan_sweep_status); every CTA still in the launch then leaves at its
// next barrier, which sees the flag or runs out its own limit.  The launch is cooperative, so the runtime refuses
// a grid whose CTAs cannot all be resident instead of letting it wait.
#include "block_body.cuh"

#include <string.h>

// Grid barrier.  Thread 0 of each CTA publishes the CTA's writes (fence after
// the CTA barrier), arrives, and waits for the generation to change; the
// fence after the wait makes the other CTAs' writes visible to this CTA's
// later loads.  Returns false when the error flag is set.
__device__ __forceinline__ bool sweep_barrier(const SweepSync& s) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vgen = s.gen;
    const unsigned g0 = *vgen;
    __threadfence();
    int good = 1;
    if (atomicAdd(s.count, 1u) + 1u == gridDim.x) {
      atomicExch(s.count, 0u);
      __threadfence();
      atomicAdd(s.gen, 1u);
    } else {
      unsigned it = 0;
      while (*vgen == g0) {
        if (++it > s.spin_limit) {
          atomicExch(s.err, 1);
          good = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    if (*(volatile int*)s.err) good = 0;
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

template <typename CT, int DMAX>
__global__ void __launch_bounds__(APPLY_THREADS, ApplyMinBlocks<DMAX>::value)
    sweep_forward_kernel(const SweepOp* __restrict__ ops, int n_ops, int store_every, const CT* state_in,
                         CT* states, int64_t slot_elems, const double2* __restrict__ arena, int D,
                         SweepSync sync) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_next[2];
  CT* Ms = reinterpret_cast<CT*>(smem_raw);
  const CT* cur = state_in;
  for (int k = 0; k < n_ops; ++k) {
    const SweepOp* op = ops + k;
    const AxisView v = op->view;
    const int layout = op->layout, mflags = op->mflags, nx = op->fwd_nx;
    const double2* mat = arena + op->m_off;
    CT* dst = states + out_slot(k, n_ops, store_every) * slot_elems;
    const int nitems = (layout == LAYOUT_DENSE ? 1 : 2 * D - 1) * nx;
    // items in block-major order (largest blocks first), taken from a per-op
    // counter: the first one by CTA index, later ones as CTAs become free;
    // the next item index is fetched while the current one is processed
    unsigned* ctr = sync.items + k;
    int it = blockIdx.x;
    int par = 0;
    if (threadIdx.x == 0) s_next[0] = gridDim.x + atomicAdd(ctr, 1u);
    while (it < nitems) {
      __syncthreads();  // s_next[par] written; Ms free for restaging
      const int next = s_next[par];
      // (a CTA whose first index is already past the end never enters this
      // loop; the index it grabbed above is >= gridDim.x > nitems, so no item
      // is lost)
      if (threadIdx.x == 0 && next < nitems) s_next[par ^ 1] = gridDim.x + atomicAdd(ctr, 1u);
      const int y = it / nx, x = it - y * nx;
      const int b = layout == LAYOUT_DENSE ? 0 : block_of_y(D, y);
      const BlockGeom g = block_geom(v, D, layout, b, (mflags & MF_SWAP) ? 1 : 0);
      const int64_t j0 = (int64_t)x * APPLY_THREADS + threadIdx.x;
      ApplyDispatch<CT, kSStep, DMAX, true>::run(cur, dst, v, D, Ms, mat, mflags, g, j0);
      it = next;
      par ^= 1;
    }
    if (!sweep_barrier(sync)) return;
    cur = dst;
  }
}

template <typename CT, int TILE, int DMAX>
__global__ void __launch_bounds__(TILE, AdjMinBlocks<CT, DMAX>::value)
    sweep_backward_kernel(const SweepOp* __restrict__ ops, int n_ops, const CT* state_in, const CT* states,
                          int64_t slot_elems, CT* lam_a, CT* lam_b, const double2* __restrict__ arena,
                          double2* cpart, double2* carena, int64_t carena_entries, int D, SweepSync sync) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  for (int i = 0; i < n_ops; ++i) {
    const int k = n_ops - 1 - i;
    const SweepOp* op = ops + k;
    const AdjSched& sc = op->sc;
    if ((int)blockIdx.x < sc.total) {
      const CT* psi_in = k == 0 ? state_in : states + (int64_t)(k - 1) * slot_elems;
      const CT* lam_out = (i & 1) ? lam_b : lam_a;
      CT* lam_in = (i & 1) ? lam_a : lam_b;
      const AxisView v = op->view;
      const int layout = op->layout, mflags = op->mflags;
      int y = 0;
      while (y + 1 < sc.nblk && (int)blockIdx.x >= sc.start[y + 1]) ++y;
      const int xrank = (int)blockIdx.x - sc.start[y];
      const int gxb = sc.gx[y];
      const int b = layout == LAYOUT_DENSE ? 0 : block_of_y(D, y);
      const BlockGeom g = block_geom(v, D, layout, b, (mflags & MF_SWAP) ? 1 : 0);
      const int s = g.s;
      const int rows = 4 * ((s + 3) / 4);
      const int bs =
          layout == LAYOUT_DENSE ? 0 : ((layout == LAYOUT_DIFF && (mflags & MF_SWAP)) ? 2 * D - 2 - b : b);
      double2* mypart = cpart + op->part_base + sc.part_off[bs] + (int64_t)xrank * s * s;
      CT* MsH = reinterpret_cast<CT*>(smem_raw);
      CT* lam_s = MsH + ((ms_slots(sizeof(CT) == 8 ? FOCK_C64 : FOCK_C128, D) + 1) & ~(size_t)1);
      CT* psi_s = lam_s + rows * (TILE + 1);
      AdjDispatch<CT, kSStep, DMAX, TILE>::run(psi_in, lam_out, lam_in, v, D, MsH, arena + op->m_off, mflags, lam_s,
                                          psi_s, g, mypart, xrank, gxb, 1);
    }
    if (!sweep_barrier(sync)) return;
  }
  // C[e] = sum over the op's CTAs x of part[x][e] for every op (one warp per
  // entry, lanes over x, fixed order)
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int k = 0;
  for (int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < carena_entries; e += nwarps) {
    while (k + 1 < n_ops && ops[k + 1].c_off <= e) ++k;
    const SweepOp* op = ops + k;
    const int layout = op->layout;
    const int64_t le = e - op->c_off;
    int bs = 0, s = D;
    int64_t off = 0;
    if (layout != LAYOUT_DENSE) {
      for (bs = 0; bs < 2 * D - 1; ++bs) {
        s = blk_size(D, bs);
        if (le < off + (int64_t)s * s) break;
        off += (int64_t)s * s;
      }
    }
    const AdjSched& sc = op->sc;
    int gxs = 1;
    for (int y = 0; y < sc.nblk; ++y)
      if ((layout == LAYOUT_DENSE ? D : blk_size(D, block_of_y(D, y))) == s) {
        gxs = sc.gx[y];
        break;
      }
    const double2* src = cpart + op->part_base + sc.part_off[bs] + (le - off);
    double2 a = make_double2(0.0, 0.0);
    for (int x = lane; x < gxs; x += 32) {
      const double2 p = src[(int64_t)x * s * s];
      a.x += p.x;
      a.y += p.y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a.x += __shfl_xor_sync(0xffffffffu, a.x, o);
      a.y += __shfl_xor_sync(0xffffffffu, a.y, o);
    }
    if (lane == 0) carena[e] = a;
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int adj_tile(int dtype) { return dtype == FOCK_C64 ? 256 : 128; }

static size_t fwd_smem(int dtype, int D) { return ms_slots(dtype, D) * (dtype == FOCK_C64 ? 8 : 16); }

static size_t bwd_smem(int dtype, int D) {
  const int esz = dtype == FOCK_C64 ? 8 : 16;
  const int rows = 4 * ((D + 3) / 4);
  return (size_t)esz * (((ms_slots(dtype, D) + 1) & ~(size_t)1) + 2 * (size_t)rows * (adj_tile(dtype) + 1));
}

template <typename K>
static int co_resident(K k, int threads, size_t smem) {
  int per_sm = 0;
  if ((smem > 48 * 1024 &&
       cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return per_sm * fock_num_sms();
}

template <typename CT, int DMAX>
static int sweep_grid_t(int dtype, int D, int backward) {
  if (backward) return co_resident(sweep_backward_kernel<CT, sizeof(CT) == 8 ? 256 : 128, DMAX>, adj_tile(dtype),
                                   bwd_smem(dtype, D));
  return co_resident(sweep_forward_kernel<CT, DMAX>, APPLY_THREADS, fwd_smem(dtype, D));
}

template <typename CT>
static int sweep_grid_d(int dtype, int D, int backward) {
  switch (dmax_bucket(D)) {
    case 4: return sweep_grid_t<CT, 4>(dtype, D, backward);
    case 8: return sweep_grid_t<CT, 8>(dtype, D, backward);
    case 12: return sweep_grid_t<CT, 12>(dtype, D, backward);
    case 16: return sweep_grid_t<CT, 16>(dtype, D, backward);
    case 20: return sweep_grid_t<CT, 20>(dtype, D, backward);
    case 24: return sweep_grid_t<CT, 24>(dtype, D, backward);
    default: return 0;
  }
}

int sweep_grid(int dtype, int D, int backward) {
  // complex64 only: complex128 ops are FP64-bound, so their launch overhead
  // matters less than the build time of another set of kernels
  if (dtype != FOCK_C64) return 0;
  int dev = 0, coop = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) {
    cudaGetLastError();
    return 0;
  }
  return sweep_grid_d<float2>(dtype, D, backward);
}

AdjSched make_adj_sched_grid(int dtype, const AxisView& v, int D, int layout, int grid) {
  AdjSched sc;
  memset(&sc, 0, sizeof(sc));
  sc.nblk = layout == LAYOUT_DENSE ? 1 : 2 * D - 1;
  if (sc.nblk > ADJ_MAX_BLOCKS) sc.nblk = 0;  // cutoff beyond FOCK_MAX_CUTOFF: callers reject it first
  const int64_t ntiles = (v.ncols + adj_tile(dtype) - 1) / adj_tile(dtype);
  // the same number of CTAs for every block, all of them within the grid
  int64_t gx = grid / sc.nblk;
  if (gx > ntiles) gx = ntiles;
  if (gx < 1) gx = 1;
  int start = 0;
  for (int y = 0; y < sc.nblk; ++y) {
    sc.gx[y] = (int)gx;
    sc.start[y] = start;
    start += (int)gx;
  }
  sc.start[sc.nblk] = start;
  sc.total = start;
  int64_t part = 0;
  for (int bs = 0; bs < sc.nblk; ++bs) {
    const int s = layout == LAYOUT_DENSE ? D : blk_size(D, bs);
    sc.part_off[bs] = part;
    part += gx * s * s;
  }
  sc.part_entries = part;
  return sc;
}

static cudaLaunchAttribute coop_attr() {
  cudaLaunchAttribute a;
  a.id = cudaLaunchAttributeCooperative;
  a.val.cooperative = 1;
  return a;
}

template <typename CT, int DMAX>
static int sweep_fwd_t(int dtype, int D, const SweepOp* ops, int n_ops, int store_every, const void* state_in,
                       void* states, int64_t slot_elems, const double2* arena, SweepSync sync, int grid,
                       cudaStream_t st) {
  auto k = sweep_forward_kernel<CT, DMAX>;
  const size_t sm = fwd_smem(dtype, D);
  if (sm > 48 * 1024) FOCK_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(APPLY_THREADS);
  cfg.dynamicSmemBytes = sm;
  cfg.stream = st;
  cudaLaunchAttribute attr = coop_attr();
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  FOCK_CUDA_TRY(cudaLaunchKernelEx(&cfg, k, ops, n_ops, store_every, (const CT*)state_in, (CT*)states, slot_elems,
                                   arena, D, sync));
  return FOCK_OK;
}

template <typename CT, int DMAX>
static int sweep_bwd_t(int dtype, int D, const SweepOp* ops, int n_ops, const void* state_in, const void* states,
                       int64_t slot_elems, void* lam_a, void* lam_b, const double2* arena, double2* cpart,
                       double2* carena, int64_t carena_entries, SweepSync sync, int grid, cudaStream_t st) {
  constexpr int TILE = sizeof(CT) == 8 ? 256 : 128;
  auto k = sweep_backward_kernel<CT, TILE, DMAX>;
  const size_t sm = bwd_smem(dtype, D);
  if (sm > 48 * 1024) FOCK_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(TILE);
  cfg.dynamicSmemBytes = sm;
  cfg.stream = st;
  cudaLaunchAttribute attr = coop_attr();
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  FOCK_CUDA_TRY(cudaLaunchKernelEx(&cfg, k, ops, n_ops, (const CT*)state_in, (const CT*)states, slot_elems,
                                   (CT*)lam_a, (CT*)lam_b, arena, cpart, carena, carena_entries, D, sync));
  return FOCK_OK;
}

#define SWEEP_DISPATCH(FN, CT, ...)                                  \
  switch (dmax_bucket(D)) {                                          \
    case 4: return FN<CT, 4>(__VA_ARGS__);                           \
    case 8: return FN<CT, 8>(__VA_ARGS__);                           \
    case 12: return FN<CT, 12>(__VA_ARGS__);                         \
    case 16: return FN<CT, 16>(__VA_ARGS__);                         \
    case 20: return FN<CT, 20>(__VA_ARGS__);                         \
    case 24: return FN<CT, 24>(__VA_ARGS__);                         \
    default: return fock_set_error(FOCK_ERR_UNSUPPORTED, "no persistent sweep for cutoff %d", D); \
  }

int launch_sweep_forward(int dtype, int D, const SweepOp* ops, int n_ops, int store_every, const void* state_in,
                         void* states, int64_t slot_elems, const double2* arena, SweepSync sync, int grid,
                         cudaStream_t st) {
  if (dtype != FOCK_C64) return fock_set_error(FOCK_ERR_UNSUPPORTED, "persistent sweeps are complex64 only");
  SWEEP_DISPATCH(sweep_fwd_t, float2, dtype, D, ops, n_ops, store_every, state_in, states, slot_elems, arena, sync,
                 grid, st)
}

int launch_sweep_backward(int dtype, int D, const SweepOp* ops, int n_ops, const void* state_in, const void* states,
                          int64_t slot_elems, void* lam_a, void* lam_b, const double2* arena, double2* cpart,
                          double2* carena, int64_t carena_entries, SweepSync sync, int grid, cudaStream_t st) {
  if (dtype != FOCK_C64) return fock_set_error(FOCK_ERR_UNSUPPORTED, "persistent sweeps are complex64 only");
  SWEEP_DISPATCH(sweep_bwd_t, float2, dtype, D, ops, n_ops, state_in, states, slot_elems, lam_a, lam_b, arena, cpart,
                 carena, carena_entries, sync, grid, st)
}
