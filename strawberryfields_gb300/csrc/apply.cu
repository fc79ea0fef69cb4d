// Gate application kernels (rows K1-K5 of the hot path).
//
// One kernel covers every non-diagonal op: a gate matrix stored as one dense
// D x D block (single-mode gates) or as 2D-1 photon-number blocks (beamsplitter
// / MZ conserve n1+n2, two-mode squeezing and the loss superoperator conserve
// n1-n2 -- the selection rules the reference exploits in
// fockbackend/circuit.py:307-365).  Grid: x over columns, y over blocks
// (largest first).  Each thread takes one column: it loads the s values of
// its block into registers (coalesced across the warp: consecutive threads
// take consecutive columns, i.e. consecutive addresses along the innermost
// non-gate axis), multiplies by the s x s block held in shared memory
// (broadcast reads) and stores s outputs.  The kernel is compiled per cutoff
// bucket DMAX so its register budget allows 4 resident CTAs (32 warps) per
// SM -- the other warps' loads hide each warp's memory latency; block sizes
// are compile-time constants through a dispatch chain, so loads and complex
// FMAs are fully unrolled.
#include "apply.cuh"

static void set_fastdiv(AxisView& v) {
  v.fast = v.ncols < ((int64_t)1 << 32);
  v.fc = make_fastdiv(v.fast ? (uint32_t)v.C : 1u);
  v.fb = make_fastdiv(v.fast ? (uint32_t)v.B : 1u);
}

AxisView make_view1(int naxes, int D, int ax) {
  AxisView v;
  int64_t C = 1;
  for (int k = ax + 1; k < naxes; ++k) C *= D;
  int64_t A = 1;
  for (int k = 0; k < ax; ++k) A *= D;
  v.A = A; v.B = 1; v.C = C; v.s1 = C; v.s2 = 0;
  v.ncols = A * C;
  set_fastdiv(v);
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
  set_fastdiv(v);
  return v;
}

#include "block_body.cuh"

template <typename CT, int DMAX>
__global__ void __launch_bounds__(APPLY_THREADS, ApplyMinBlocks<DMAX>::value) apply_block_kernel(
    const CT* __restrict__ in, CT* __restrict__ out, AxisView v, int D, int layout, const double2* __restrict__ mat,
    int mflags, BatchArg bt, int il) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CT* Ms = reinterpret_cast<CT*>(smem_raw);
  in += blockIdx.z * bt.state_stride;
  out += blockIdx.z * bt.state_stride;
  mat = mat_batch(mat, blockIdx.z * bt.mat_stride, mflags);
  // grid (column tiles, blocks) or, interleaved (il), (blocks, column tiles)
  const int yb = il ? (int)blockIdx.x : (int)blockIdx.y;
  const int64_t tile = il ? (int64_t)blockIdx.y : (int64_t)blockIdx.x;
  const int b = layout == LAYOUT_DENSE ? 0 : block_of_y(D, yb);
  const BlockGeom g = block_geom(v, D, layout, b, (mflags & MF_SWAP) ? 1 : 0);
  const int64_t j0 = tile * (APPLY_THREADS * APPLY_COLS) + threadIdx.x;
  // the matrix was built before the sweep: stage it while the previous op
  // finishes
  StageDispatch<CT, kSStep, DMAX>::run(Ms, mat, g, mflags);
  pdl_wait();
  pdl_launch_dependents();
  ApplyDispatch<CT, kSStep, DMAX>::run(in, out, v, D, Ms, mat, mflags, g, j0, 1);
}

template <typename CT, int DMAX>
static int launch_apply_t(const void* in, void* out, const AxisView& v, int D, int layout, const double2* mat,
                          int mflags, cudaStream_t st, const BatchArg& bt) {
  const int nblk = layout == LAYOUT_DENSE ? 1 : 2 * D - 1;
  const int64_t gx = (v.ncols + APPLY_THREADS * APPLY_COLS - 1) / (APPLY_THREADS * APPLY_COLS);
  if (gx > 0x7fffffffLL) return fock_set_error(FOCK_ERR_INVALID, "state too large");
  if (bt.nb < 1 || bt.nb > 65535) return fock_set_error(FOCK_ERR_INVALID, "batch of %d circuits", bt.nb);
  // blocks of one column tile next to each other when they share sectors
  const bool il = interleave_blocks(layout, v) && gx > 1 && gx <= 65535;
  dim3 grid(il ? (unsigned)nblk : (unsigned)gx, il ? (unsigned)gx : (unsigned)nblk, bt.nb);
  const size_t sm = ms_slots(sizeof(CT) == 8 ? FOCK_C64 : FOCK_C128, D) * sizeof(CT);
  auto k = apply_block_kernel<CT, DMAX>;
  if (sm > 48 * 1024) FOCK_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  FOCK_CUDA_TRY(launch_kernel(k, grid, dim3(APPLY_THREADS), sm, st, bt.pdl, (const CT*)in, (CT*)out, v, D, layout,
                               mat, mflags, bt, (int)il));
  return FOCK_OK;
}

template <typename CT>
static int launch_apply_d(const void* in, void* out, const AxisView& v, int D, int layout, const double2* mat,
                          int mflags, cudaStream_t st, const BatchArg& bt) {
  switch (dmax_bucket(D)) {
    case 4: return launch_apply_t<CT, 4>(in, out, v, D, layout, mat, mflags, st, bt);
    case 8: return launch_apply_t<CT, 8>(in, out, v, D, layout, mat, mflags, st, bt);
    case 12: return launch_apply_t<CT, 12>(in, out, v, D, layout, mat, mflags, st, bt);
    case 16: return launch_apply_t<CT, 16>(in, out, v, D, layout, mat, mflags, st, bt);
    case 20: return launch_apply_t<CT, 20>(in, out, v, D, layout, mat, mflags, st, bt);
    case 24: return launch_apply_t<CT, 24>(in, out, v, D, layout, mat, mflags, st, bt);
    default: return launch_apply_t<CT, 0>(in, out, v, D, layout, mat, mflags, st, bt);
  }
}

int launch_apply(int dtype, const void* in, void* out, const AxisView& v, int D, int layout,
                 const double2* mat, int mflags, cudaStream_t st, const BatchArg& bt) {
  if (v.ncols <= 0) return FOCK_OK;
  if (dtype == FOCK_C64) return launch_apply_d<float2>(in, out, v, D, layout, mat, mflags, st, bt);
  return launch_apply_d<double2>(in, out, v, D, layout, mat, mflags, st, bt);
}
