// Adding and removing modes of a state on the device.
//
// fock_append_vacuum: |psi> -> |psi> (x) |0...0> with the new modes last
// (Circuit.alloc, strawberryfields/backends/fockbackend/circuit.py:373-382).
// fock_partial_trace: rho -> Tr_modes rho for a density matrix with
// interleaved (ket, bra) axes, the kept modes staying in their order
// (Circuit.dealloc :384-391 through ops.partial_trace, fockbackend/ops.py:144).
// Neither is on a sweep's hot path: one write pass (append) and one read pass
// over the diagonal slices of the traced modes (trace), FP64 accumulation.
#include "fock_common.cuh"

namespace {

constexpr int kMaxTraceModes = FOCK_MAX_AXES / 2;

int state_elems(int naxes, int D, int64_t* n) {
  if (D < 1 || D > FOCK_MAX_CUTOFF)
    return fock_set_error(FOCK_ERR_INVALID, "cutoff must be in [1, %d], got %d", FOCK_MAX_CUTOFF, D);
  if (naxes < 0 || naxes > FOCK_MAX_AXES)
    return fock_set_error(FOCK_ERR_INVALID, "too many axes (%d)", naxes);
  if (naxes * log2((double)D) > 60.0)
    return fock_set_error(FOCK_ERR_INVALID, "state of %d^%d entries is too large", D, naxes);
  int64_t e = 1;
  for (int k = 0; k < naxes; ++k) e *= D;
  *n = e;
  return FOCK_OK;
}

unsigned grid_1d(int64_t n) {
  int64_t g = (n + 255) / 256;
  if (g > 152 * 32) g = 152 * 32;
  return (unsigned)(g < 1 ? 1 : g);
}

template <typename CT>
__global__ void append_vacuum_kernel(const CT* __restrict__ in, CT* __restrict__ out, int64_t n_out,
                                     int64_t stride) {
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n_out; j += step) {
    const int64_t q = j / stride;
    out[j] = (j == q * stride) ? in[q] : czero<CT>();
  }
}

struct TraceArgs {
  int D, nk, nt;
  int64_t kept_sk[kMaxTraceModes];  // input stride of each kept mode's ket axis
  int64_t kept_sb[kMaxTraceModes];  // ... and of its bra axis
  int64_t tr_s[kMaxTraceModes];     // input step along a traced mode's diagonal
  int64_t n_traces;                 // D^nt
};

template <typename CT>
__global__ void partial_trace_kernel(const CT* __restrict__ rho, CT* __restrict__ out, int64_t n_out,
                                     TraceArgs a) {
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < n_out; o += step) {
    int64_t r = o, base = 0;
    for (int i = a.nk - 1; i >= 0; --i) {
      const int64_t b = r % a.D;
      r /= a.D;
      const int64_t k = r % a.D;
      r /= a.D;
      base += k * a.kept_sk[i] + b * a.kept_sb[i];
    }
    double re = 0.0, im = 0.0;
    for (int64_t t = 0; t < a.n_traces; ++t) {
      int64_t tt = t, off = base;
      for (int j = a.nt - 1; j >= 0; --j) {
        off += (tt % a.D) * a.tr_s[j];
        tt /= a.D;
      }
      const CT v = rho[off];
      re += (double)v.x;
      im += (double)v.y;
    }
    CT w;
    w.x = re;
    w.y = im;
    out[o] = w;
  }
}

}  // namespace

extern "C" int fock_append_vacuum(int num_modes, int n_new, int cutoff, int pure, int dtype, const void* in,
                                  void* out, void* stream) {
  if (dtype != FOCK_C64 && dtype != FOCK_C128)
    return fock_set_error(FOCK_ERR_INVALID, "dtype must be FOCK_C64 or FOCK_C128");
  if (num_modes < 1 || n_new < 1)
    return fock_set_error(FOCK_ERR_INVALID, "need at least one mode and one new mode (got %d, %d)", num_modes,
                          n_new);
  const int per = pure ? 1 : 2;
  int64_t n_out = 0, stride = 0;
  int rc = state_elems(per * (num_modes + n_new), cutoff, &n_out);
  if (rc) return rc;
  if ((rc = state_elems(per * n_new, cutoff, &stride))) return rc;
  if (!in || !out) return fock_set_error(FOCK_ERR_INVALID, "null state buffer");
  if (in == out) return fock_set_error(FOCK_ERR_INVALID, "in and out must be different buffers");
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == FOCK_C64)
    append_vacuum_kernel<float2><<<grid_1d(n_out), 256, 0, st>>>((const float2*)in, (float2*)out, n_out, stride);
  else
    append_vacuum_kernel<double2><<<grid_1d(n_out), 256, 0, st>>>((const double2*)in, (double2*)out, n_out,
                                                                   stride);
  FOCK_LAUNCH_CHECK("append_vacuum_kernel");
  return FOCK_OK;
}

extern "C" int fock_partial_trace(int num_modes, int cutoff, int dtype, int n_traced, const int* modes,
                                  const void* rho, void* out, void* stream) {
  if (dtype != FOCK_C64 && dtype != FOCK_C128)
    return fock_set_error(FOCK_ERR_INVALID, "dtype must be FOCK_C64 or FOCK_C128");
  if (num_modes < 1 || num_modes > kMaxTraceModes)
    return fock_set_error(FOCK_ERR_INVALID, "number of modes must be in [1, %d], got %d", kMaxTraceModes,
                          num_modes);
  if (n_traced < 1 || n_traced >= num_modes || !modes)
    return fock_set_error(FOCK_ERR_INVALID, "trace over 1 to %d of the %d modes (got %d)", num_modes - 1,
                          num_modes, n_traced);
  int64_t n_in = 0, n_out = 0, n_tr = 0;
  int rc = state_elems(2 * num_modes, cutoff, &n_in);
  if (rc) return rc;
  state_elems(2 * (num_modes - n_traced), cutoff, &n_out);
  state_elems(n_traced, cutoff, &n_tr);
  if (!rho || !out) return fock_set_error(FOCK_ERR_INVALID, "null state buffer");
  if (rho == out) return fock_set_error(FOCK_ERR_INVALID, "rho and out must be different buffers");
  bool traced[kMaxTraceModes] = {false};
  for (int i = 0; i < n_traced; ++i) {
    if (modes[i] < 0 || modes[i] >= num_modes)
      return fock_set_error(FOCK_ERR_INVALID, "mode %d is not a valid mode of a %d-mode state", modes[i],
                            num_modes);
    if (traced[modes[i]]) return fock_set_error(FOCK_ERR_INVALID, "mode %d is listed twice", modes[i]);
    traced[modes[i]] = true;
  }
  TraceArgs a;
  a.D = cutoff;
  a.nk = num_modes - n_traced;
  a.nt = n_traced;
  a.n_traces = n_tr;
  int ik = 0, it = 0;
  for (int m = 0; m < num_modes; ++m) {
    int64_t sb = 1;
    for (int k = 0; k < 2 * (num_modes - 1 - m); ++k) sb *= cutoff;
    const int64_t sk = sb * cutoff;
    if (traced[m]) {
      a.tr_s[it++] = sk + sb;
    } else {
      a.kept_sk[ik] = sk;
      a.kept_sb[ik++] = sb;
    }
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == FOCK_C64)
    partial_trace_kernel<float2><<<grid_1d(n_out), 256, 0, st>>>((const float2*)rho, (float2*)out, n_out, a);
  else
    partial_trace_kernel<double2><<<grid_1d(n_out), 256, 0, st>>>((const double2*)rho, (double2*)out, n_out, a);
  FOCK_LAUNCH_CHECK("partial_trace_kernel");
  return FOCK_OK;
}
