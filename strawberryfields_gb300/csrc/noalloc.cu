// Single-mode reduced density matrix without any device allocation.
//
// Some callers cannot allocate device memory at all: code running inside a
// host callback or a real-time loop where cudaMalloc would stall or is
// forbidden, processes whose memory is owned by another allocator (a
// framework pool), and plain-C hosts that only hold the state buffer.  The
// regular fock_reduced_dm1 needs a caller-provided workspace for the per-CTA
// partial sums of its reduction; this variant keeps that scratch in a
// fixed-size array in device global memory that lives as long as the library
// is loaded (every GPU that loads the library holds it until exit).
#include "apply.cuh"

#include <mutex>

#define FOCK_NOALLOC_SCRATCH_BYTES (512 * 1024)
#define FOCK_NOALLOC_MIN_SLOTS 8

// Largest cutoff D whose D*D complex128 slots fit the scratch FOCK_NOALLOC_MIN_SLOTS
// times after the one slot of the reduced contraction.
static constexpr int noalloc_max_cutoff() {
  int d = 1;
  while ((int64_t)16 * (d + 1) * (d + 1) * (FOCK_NOALLOC_MIN_SLOTS + 1) <= FOCK_NOALLOC_SCRATCH_BYTES) ++d;
  return d;
}
static_assert(noalloc_max_cutoff() == FOCK_NOALLOC_MAX_CUTOFF,
              "FOCK_NOALLOC_MAX_CUTOFF in fock_gb300.h must match the scratch size");

static __device__ __align__(256) unsigned char g_noalloc_scratch[FOCK_NOALLOC_SCRATCH_BYTES];

// In host code `g_noalloc_scratch` names a host-side stand-in, not a device
// address: the device address is looked up with the device current.  Outside
// stream capture it is looked up on every call (cheap, and right after a
// cudaDeviceReset or under a different context); while `stream` is capturing,
// the address cached by the last uncaptured call on this device is used.
static void* g_scratch_dev[64] = {nullptr};
static std::mutex g_scratch_mu;

static int noalloc_scratch(cudaStream_t stream, double2** out) {
  int dev = 0;
  FOCK_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fock_set_error(FOCK_ERR_INVALID, "device index %d out of range", dev);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess) {
    cudaGetLastError();  // clear it; treat as capturing (use the cached address)
    cap = cudaStreamCaptureStatusActive;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_dev[dev] || cap == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return fock_check_cuda(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_scratch_dev[dev] = p;
  }
  *out = (double2*)g_scratch_dev[dev];
  return FOCK_OK;
}

extern "C" int fock_reduced_dm1_noalloc(int num_modes, int cutoff, int pure, int dtype, int mode,
                                        const void* state, void* out, void* stream) {
  int rc = check_reduced_dm1_args(num_modes, cutoff, pure, dtype, mode, state, out);
  if (rc) return rc;
  const int D = cutoff;
  const int64_t slot_bytes = (int64_t)D * D * sizeof(double2);
  // one slot for the reduced contraction, the rest for per-CTA partial sums
  const int64_t slots = FOCK_NOALLOC_SCRATCH_BYTES / slot_bytes - 1;
  if (slots < FOCK_NOALLOC_MIN_SLOTS)
    return fock_set_error(FOCK_ERR_INVALID,
                          "cutoff %d is too large for the fixed %d-byte scratch of fock_reduced_dm1_noalloc "
                          "(largest cutoff: %d); use fock_reduced_dm1 with a caller-provided workspace",
                          D, FOCK_NOALLOC_SCRATCH_BYTES, noalloc_max_cutoff());
  cudaStream_t st = (cudaStream_t)stream;
  double2* scratch = nullptr;
  if ((rc = noalloc_scratch(st, &scratch))) return rc;
  if (pure) {
    // C[u][v] = sum conj(psi[u]) psi[v] = rho[v][u]; every partial slot the
    // grid uses is written before it is read, so nothing needs clearing
    AxisView v = make_view1(num_modes, D, mode);
    AdjSched sc = make_adj_sched(dtype, v, D, LAYOUT_DENSE);
    if (sc.gx[0] > slots) {
      // fewer CTAs, each covering more column tiles, so the partials fit
      sc.gx[0] = (int)slots;
      sc.start[1] = sc.total = (int)slots;
      sc.part_entries = slots * (int64_t)D * D;
    }
    double2* C = scratch;
    double2* cpart = scratch + (int64_t)D * D;
    rc = launch_adjoint_partials(dtype, state, state, nullptr, v, D, LAYOUT_DENSE, C, 0, cpart, sc, st);
    if (rc) return rc;
    if ((rc = launch_reduce_sched(cpart, sc, D, LAYOUT_DENSE, C, st))) return rc;
    return launch_transpose_dm(C, (double2*)out, D, st);
  }
  int64_t ntr = 1;
  for (int k = 0; k < num_modes - 1; ++k) ntr *= D;
  int64_t chunks = (ntr + 4095) / 4096;
  if (chunks > 64) chunks = 64;
  // defensive: ntr = D^(n-1) > 4096 * slots needs a density matrix far larger
  // than device memory at every accepted cutoff, so this cap never binds
  if (chunks > slots) chunks = slots;
  if (chunks < 1) chunks = 1;
  rc = launch_rdm_mixed(dtype, state, num_modes, D, mode, ntr, (int)chunks, scratch, st);
  if (rc) return rc;
  return launch_reduce_partials(scratch, (int)chunks, (int64_t)D * D, (double2*)out, st);
}
