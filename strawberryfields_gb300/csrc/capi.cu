// C ABI entry points for single operations: error state, gate application,
// diagonal phases, mix, vacuum, mode preparation and readouts.
#include "apply.cuh"

#include <stdarg.h>
#include <stdio.h>
#include <string.h>

static thread_local char g_err[1024] = "";

int fock_set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

int fock_check_cuda(cudaError_t e, const char* what) {
  // a failed runtime call also sets the thread's last CUDA error; read it
  // here so a later launch check does not report this failure again (a
  // sticky error, after a device fault, stays set regardless)
  cudaGetLastError();
  return fock_set_error(FOCK_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

extern "C" int fock_last_error(char* buf, size_t len) {
  size_t n = strlen(g_err);
  if (buf && len) {
    size_t c = n < len - 1 ? n : len - 1;
    memcpy(buf, g_err, c);
    buf[c] = 0;
  }
  return (int)n;
}

extern "C" int fock_version(void) { return 1; }

int fock_num_sms() {
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  if (!cache[dev]) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
    cache[dev] = n;
  }
  return cache[dev];
}

static inline int esize(int dtype) { return dtype == FOCK_C64 ? 8 : 16; }

// validate a state description; returns element count via *elems
static int check_state(int num_modes, int cutoff, int pure, int dtype, int64_t* elems) {
  if (dtype != FOCK_C64 && dtype != FOCK_C128) return fock_set_error(FOCK_ERR_INVALID, "dtype must be FOCK_C64 or FOCK_C128");
  if (cutoff < 1 || cutoff > FOCK_MAX_CUTOFF)
    return fock_set_error(FOCK_ERR_INVALID, "cutoff must be in [1, %d], got %d", FOCK_MAX_CUTOFF, cutoff);
  if (num_modes < 1) return fock_set_error(FOCK_ERR_INVALID, "number of modes must be positive, got %d", num_modes);
  const int naxes = pure ? num_modes : 2 * num_modes;
  if (naxes > FOCK_MAX_AXES) return fock_set_error(FOCK_ERR_INVALID, "too many modes (%d)", num_modes);
  double lg = naxes * log2((double)cutoff);
  if (lg > 60.0) return fock_set_error(FOCK_ERR_INVALID, "state of %d^%d entries is too large", cutoff, naxes);
  int64_t n = 1;
  for (int k = 0; k < naxes; ++k) n *= cutoff;
  if (elems) *elems = n;
  return FOCK_OK;
}

static int check_mode(int m, int num_modes, const char* what) {
  if (m < 0 || m >= num_modes)
    return fock_set_error(FOCK_ERR_INVALID, "%s %d is not a valid mode of a %d-mode state", what, m, num_modes);
  return FOCK_OK;
}

// view of one or two modes: sorted axes, swap flag
static AxisView mode_view(int naxes, int D, int a1, int a2, int* swap) {
  *swap = 0;
  if (a2 < 0) return make_view1(naxes, D, a1);
  if (a1 > a2) { int t = a1; a1 = a2; a2 = t; *swap = 1; }
  return make_view2(naxes, D, a1, a2);
}

// apply an already-built matrix (layout) to a pure or mixed state
// out = M in on one view: the plane-tile kernel for the ops it is preferred
// for, else the block-per-CTA kernel
static int apply_view(int dtype, const void* in, void* out, const AxisView& v, int D, int layout,
                      const double2* M, int mflags, cudaStream_t st) {
  PlaneGeom g;
  if (plane_preferred(layout, v) && make_plane_geom(dtype, v, D, layout, (mflags & MF_SWAP) ? 1 : 0, 0, &g))
    return launch_plane_apply(dtype, in, out, g, plane_grid(dtype, g, 0, 1), M, mflags, st);
  return launch_apply(dtype, in, out, v, D, layout, M, mflags, st);
}

static int apply_built(const double2* M, int layout, int mode1, int mode2, int num_modes, int D, int pure,
                       int dtype, const void* in, void* out, void* tmp, int is_channel, cudaStream_t st) {
  int swap = 0;
  if (pure) {
    AxisView v = mode_view(num_modes, D, mode1, layout == LAYOUT_DENSE ? -1 : mode2, &swap);
    return apply_view(dtype, in, out, v, D, layout, M, swap ? MF_SWAP : 0, st);
  }
  const int naxes = 2 * num_modes;
  if (is_channel) {
    // superoperator on the (ket, bra) axis pair of one mode
    AxisView v = make_view2(naxes, D, 2 * mode1, 2 * mode1 + 1);
    return apply_view(dtype, in, out, v, D, layout, M, 0, st);
  }
  if (!tmp) return fock_set_error(FOCK_ERR_INVALID, "mixed states need a temporary state buffer");
  int rc;
  if (layout == LAYOUT_DENSE) {
    AxisView vk = make_view1(naxes, D, 2 * mode1);
    rc = apply_view(dtype, in, tmp, vk, D, layout, M, 0, st);
    if (rc) return rc;
    AxisView vb = make_view1(naxes, D, 2 * mode1 + 1);
    return apply_view(dtype, tmp, out, vb, D, layout, M, MF_CONJ, st);
  }
  AxisView vk = mode_view(naxes, D, 2 * mode1, 2 * mode2, &swap);
  rc = apply_view(dtype, in, tmp, vk, D, layout, M, swap ? MF_SWAP : 0, st);
  if (rc) return rc;
  AxisView vb = mode_view(naxes, D, 2 * mode1 + 1, 2 * mode2 + 1, &swap);
  return apply_view(dtype, tmp, out, vb, D, layout, M, MF_CONJ | (swap ? MF_SWAP : 0), st);
}

// ---------------------------------------------------------------------------
// diagonal phases
// ---------------------------------------------------------------------------
#define MAX_CK 32
#define MAX_PHASE_MODES (FOCK_MAX_AXES / 2)
struct PhaseArgs {
  int naxes, D, pure, nmodes, n_ck;
  int cka[MAX_CK], ckb[MAX_CK];
  double ckk[MAX_CK];
  double theta[MAX_PHASE_MODES];  // rotation angle per mode  (theta * n)
  double kappa[MAX_PHASE_MODES];  // Kerr strength per mode   (kappa * n^2)
};

template <typename CT>
__global__ void phases_kernel(const CT* __restrict__ in, CT* __restrict__ out, int64_t n,
                              const double* __restrict__ angles, PhaseArgs P) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (int64_t)gridDim.x * blockDim.x) {
    // digits, last axis fastest
    int dig[FOCK_MAX_AXES];
    int64_t t = idx;
    for (int k = P.naxes - 1; k >= 0; --k) {
      dig[k] = (int)(t % P.D);
      t /= P.D;
    }
    double ang = 0.0;
    const int stride = P.pure ? 1 : 2;
    for (int m = 0; m < P.nmodes; ++m) {
      const double nk = dig[stride * m];
      ang += P.theta[m] * nk + P.kappa[m] * nk * nk;
      if (angles) ang += angles[m * P.D + dig[stride * m]];
      if (!P.pure) {
        const double nb = dig[2 * m + 1];
        ang -= P.theta[m] * nb + P.kappa[m] * nb * nb;
        if (angles) ang -= angles[m * P.D + dig[2 * m + 1]];
      }
    }
    for (int c = 0; c < P.n_ck; ++c) {
      ang += P.ckk[c] * (double)dig[stride * P.cka[c]] * dig[stride * P.ckb[c]];
      if (!P.pure) ang -= P.ckk[c] * (double)dig[2 * P.cka[c] + 1] * dig[2 * P.ckb[c] + 1];
    }
    double s, c;
    sincos(ang, &s, &c);
    double2 x = to_d(in[idx]);
    double2 y = make_double2(x.x * c - x.y * s, x.x * s + x.y * c);
    out[idx] = to_c(y, (CT*)nullptr);
  }
}

static unsigned grid_for(int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  int64_t cap = (int64_t)fock_num_sms() * 16;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (unsigned)g;
}

static int phase_args_init(PhaseArgs* P, int num_modes, int cutoff, int pure) {
  memset(P, 0, sizeof(*P));
  if (num_modes > MAX_PHASE_MODES) return fock_set_error(FOCK_ERR_INVALID, "too many modes");
  P->naxes = pure ? num_modes : 2 * num_modes;
  P->D = cutoff;
  P->pure = pure;
  P->nmodes = num_modes;
  return FOCK_OK;
}

static int launch_phases(const PhaseArgs& P, int dtype, int64_t n, const double* angles, const void* in,
                         void* out, cudaStream_t st) {
  if (dtype == FOCK_C64)
    phases_kernel<float2><<<grid_for(n, 256), 256, 0, st>>>((const float2*)in, (float2*)out, n, angles, P);
  else
    phases_kernel<double2><<<grid_for(n, 256), 256, 0, st>>>((const double2*)in, (double2*)out, n, angles, P);
  FOCK_LAUNCH_CHECK("phases_kernel");
  return FOCK_OK;
}


extern "C" int fock_apply_gate(int kind, double p0, double p1, int mode1, int mode2, int num_modes,
                               int cutoff, int pure, int dtype, const double* pre, const void* in,
                               void* out, void* tmp, void* workspace, void* stream) {
  int64_t n;
  int rc = check_state(num_modes, cutoff, pure, dtype, &n);
  if (rc) return rc;
  if ((rc = check_mode(mode1, num_modes, "mode"))) return rc;
  const int layout = gate_layout(kind);
  if (!layout) return fock_set_error(FOCK_ERR_INVALID, "unknown gate kind %d", kind);
  const int two = (kind == FOCK_BEAMSPLITTER || kind == FOCK_MZGATE || kind == FOCK_CROSS_KERR ||
                   kind == FOCK_TWO_MODE_SQUEEZE);
  if (two) {
    if ((rc = check_mode(mode2, num_modes, "mode"))) return rc;
    if (mode1 == mode2) return fock_set_error(FOCK_ERR_INVALID, "two-mode gate needs two distinct modes");
  }
  if (!in || !out || in == out) return fock_set_error(FOCK_ERR_INVALID, "need distinct input and output buffers");
  cudaStream_t st = (cudaStream_t)stream;
  if (kind == FOCK_LOSS && pure)
    return fock_set_error(FOCK_ERR_INVALID, "the loss channel acts on mixed states; mix the state first");
  if (kind == FOCK_ROTATION || kind == FOCK_KERR || kind == FOCK_CROSS_KERR) {
    // diagonal gates (and any pending pre-phases): one phase pass
    PhaseArgs P;
    rc = phase_args_init(&P, num_modes, cutoff, pure);
    if (rc) return rc;
    if (pre) {
      P.theta[mode1] += pre[0];
      P.kappa[mode1] += pre[1];
      if (two) { P.theta[mode2] += pre[2]; P.kappa[mode2] += pre[3]; }
    }
    if (kind == FOCK_ROTATION) P.theta[mode1] += p0;
    else if (kind == FOCK_KERR) P.kappa[mode1] += p0;
    else { P.n_ck = 1; P.cka[0] = mode1; P.ckb[0] = mode2; P.ckk[0] = p0; }
    return launch_phases(P, dtype, n, nullptr, in, out, st);
  }
  if (!workspace) return fock_set_error(FOCK_ERR_INVALID, "workspace required");
  const int64_t ne = layout_entries(layout, cutoff);
  double2* M = (double2*)workspace;
  double2* X = build_scratch_entries(kind, cutoff) > 0 ? M + ne : nullptr;
  PhaseTerm terms[6];
  int nt = 0;
  if (kind == FOCK_MZGATE) {
    // MZ(phi_in, phi_ex): external phase R(phi_ex) on mode1 acts first
    terms[nt++] = PhaseTerm{FN_A, 0, -1, 0, p1};
  }
  if (pre) {
    if (pre[0] != 0.0) terms[nt++] = PhaseTerm{FN_A, 0, -1, 0, pre[0]};
    if (pre[1] != 0.0) terms[nt++] = PhaseTerm{FN_A2, 0, -1, 0, pre[1]};
    if (two && pre[2] != 0.0) terms[nt++] = PhaseTerm{FN_B, 0, -1, 0, pre[2]};
    if (two && pre[3] != 0.0) terms[nt++] = PhaseTerm{FN_B2, 0, -1, 0, pre[3]};
    if (!two && (pre[2] != 0.0 || pre[3] != 0.0))
      return fock_set_error(FOCK_ERR_INVALID, "second-mode pre-phases given for a single-mode gate");
  }
  rc = build_single(kind, layout, cutoff, p0, p1, terms, nt, M, nullptr, X, st);
  if (rc) return rc;
  return apply_built(M, layout, mode1, two ? mode2 : -1, num_modes, cutoff, pure, dtype, in, out, tmp,
                     kind == FOCK_LOSS, st);
}

extern "C" int fock_apply_matrix1(const void* mat, int mode, int num_modes, int cutoff, int pure, int dtype,
                                  const void* in, void* out, void* tmp, void* stream) {
  int64_t n;
  int rc = check_state(num_modes, cutoff, pure, dtype, &n);
  if (rc) return rc;
  if ((rc = check_mode(mode, num_modes, "mode"))) return rc;
  if (!mat || !in || !out || in == out) return fock_set_error(FOCK_ERR_INVALID, "bad buffers");
  return apply_built((const double2*)mat, LAYOUT_DENSE, mode, -1, num_modes, cutoff, pure, dtype, in, out, tmp,
                     0, (cudaStream_t)stream);
}

extern "C" int fock_apply_phases(int num_modes, int cutoff, int pure, int dtype, const double* angles,
                                 int n_ck, const int* ck_modes, const double* ck_kappa, const void* in,
                                 void* out, void* stream) {
  int64_t n;
  int rc = check_state(num_modes, cutoff, pure, dtype, &n);
  if (rc) return rc;
  if (n_ck < 0 || n_ck > MAX_CK) return fock_set_error(FOCK_ERR_INVALID, "at most %d cross-Kerr pairs", MAX_CK);
  if (!in || !out) return fock_set_error(FOCK_ERR_INVALID, "null state buffer");
  PhaseArgs P;
  if ((rc = phase_args_init(&P, num_modes, cutoff, pure))) return rc;
  P.n_ck = n_ck;
  for (int c = 0; c < n_ck; ++c) {
    if ((rc = check_mode(ck_modes[2 * c], num_modes, "cross-Kerr mode"))) return rc;
    if ((rc = check_mode(ck_modes[2 * c + 1], num_modes, "cross-Kerr mode"))) return rc;
    P.cka[c] = ck_modes[2 * c];
    P.ckb[c] = ck_modes[2 * c + 1];
    P.ckk[c] = ck_kappa[c];
  }
  return launch_phases(P, dtype, n, angles, in, out, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// mix, vacuum
// ---------------------------------------------------------------------------
template <typename CT>
__global__ void mix_kernel(const CT* __restrict__ ket, CT* __restrict__ dm, int64_t n, int N, int D) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t t = idx, k = 0, b = 0, w = 1;
    for (int m = N - 1; m >= 0; --m) {
      int db = (int)(t % D); t /= D;
      int dk = (int)(t % D); t /= D;
      k += dk * w;
      b += db * w;
      w *= D;
    }
    dm[idx] = cmul(ket[k], cconj(ket[b]));
  }
}

extern "C" int fock_mix(int num_modes, int cutoff, int dtype, const void* ket, void* dm, void* stream) {
  int64_t n;
  int rc = check_state(num_modes, cutoff, 0, dtype, &n);
  if (rc) return rc;
  if (!ket || !dm) return fock_set_error(FOCK_ERR_INVALID, "null state buffer");
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == FOCK_C64)
    mix_kernel<float2><<<grid_for(n, 256), 256, 0, st>>>((const float2*)ket, (float2*)dm, n, num_modes, cutoff);
  else
    mix_kernel<double2><<<grid_for(n, 256), 256, 0, st>>>((const double2*)ket, (double2*)dm, n, num_modes, cutoff);
  FOCK_LAUNCH_CHECK("mix_kernel");
  return FOCK_OK;
}

__global__ void set_one_kernel(void* p, int dtype) {
  if (dtype == FOCK_C64) *(float2*)p = make_float2(1.f, 0.f);
  else *(double2*)p = make_double2(1.0, 0.0);
}

extern "C" int fock_vacuum(int num_modes, int cutoff, int pure, int dtype, void* state, void* stream) {
  int64_t n;
  int rc = check_state(num_modes, cutoff, pure, dtype, &n);
  if (rc) return rc;
  if (!state) return fock_set_error(FOCK_ERR_INVALID, "null state buffer");
  cudaStream_t st = (cudaStream_t)stream;
  FOCK_CUDA_TRY(cudaMemsetAsync(state, 0, n * esize(dtype), st));
  set_one_kernel<<<1, 1, 0, st>>>(state, dtype);
  FOCK_LAUNCH_CHECK("set_one_kernel");
  return FOCK_OK;
}

// ---------------------------------------------------------------------------
// mode preparation on mixed states: out = tr_modes(in) (x) sub
// ---------------------------------------------------------------------------
struct PrepArgs {
  int N, D, nsub;
  int is_sub[FOCK_MAX_AXES / 2];  // mode -> position in sub, or -1
};

template <typename CT>
__global__ void partial_trace_kernel(const CT* __restrict__ in, CT* __restrict__ red, int64_t nred,
                                     int64_t ntrace, PrepArgs P) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nred; r += (int64_t)gridDim.x * blockDim.x) {
    // red digits: interleaved (ket, bra) of the kept modes in order
    int kd[FOCK_MAX_AXES / 2], bd[FOCK_MAX_AXES / 2];
    int64_t t = r;
    for (int m = P.N - 1; m >= 0; --m) {
      if (P.is_sub[m] >= 0) continue;
      bd[m] = (int)(t % P.D); t /= P.D;
      kd[m] = (int)(t % P.D); t /= P.D;
    }
    double2 acc = make_double2(0.0, 0.0);
    for (int64_t k = 0; k < ntrace; ++k) {
      int64_t tt = k;
      int64_t off = 0;
      // build offset with traced modes on the diagonal
      int64_t w = 1;
      int trd[FOCK_MAX_AXES / 2];
      for (int m = P.N - 1; m >= 0; --m) {
        if (P.is_sub[m] < 0) continue;
        trd[m] = (int)(tt % P.D); tt /= P.D;
      }
      for (int m = P.N - 1; m >= 0; --m) {
        int a = P.is_sub[m] >= 0 ? trd[m] : kd[m];
        int b = P.is_sub[m] >= 0 ? trd[m] : bd[m];
        off += b * w; w *= P.D;
        off += a * w; w *= P.D;
      }
      acc = cadd(acc, to_d(in[off]));
    }
    red[r] = to_c(acc, (CT*)nullptr);
  }
}

template <typename CT>
__global__ void tensor_insert_kernel(const CT* __restrict__ red, const double2* __restrict__ sub,
                                     CT* __restrict__ out, int64_t n, PrepArgs P) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (int64_t)gridDim.x * blockDim.x) {
    int kd[FOCK_MAX_AXES / 2], bd[FOCK_MAX_AXES / 2];
    int64_t t = idx;
    for (int m = P.N - 1; m >= 0; --m) {
      bd[m] = (int)(t % P.D); t /= P.D;
      kd[m] = (int)(t % P.D); t /= P.D;
    }
    int64_t roff = 0, soff = 0, w = 1;
    for (int m = P.N - 1; m >= 0; --m) {
      if (P.is_sub[m] >= 0) continue;
      roff += bd[m] * w; w *= P.D;
      roff += kd[m] * w; w *= P.D;
    }
    // sub digits ordered by sub position: position p holds mode m with is_sub[m] == p
    w = 1;
    for (int p = P.nsub - 1; p >= 0; --p) {
      int m = 0;
      for (int q = 0; q < P.N; ++q) if (P.is_sub[q] == p) m = q;
      soff += bd[m] * w; w *= P.D;
      soff += kd[m] * w; w *= P.D;
    }
    double2 y = cmul(to_d(red[roff]), sub[soff]);
    out[idx] = to_c(y, (CT*)nullptr);
  }
}

extern "C" int64_t fock_prepare_workspace_bytes(int num_modes, int cutoff, int dtype, int n_sub) {
  if (n_sub >= num_modes) return 16;
  int64_t n = 1;
  for (int k = 0; k < 2 * (num_modes - n_sub); ++k) n *= cutoff;
  return n * esize(dtype) + 256;
}

extern "C" int fock_prepare_modes(int num_modes, int cutoff, int dtype, int n_sub, const int* modes,
                                  const void* sub, const void* in, void* out, void* workspace, void* stream) {
  int64_t n;
  int rc = check_state(num_modes, cutoff, 0, dtype, &n);
  if (rc) return rc;
  if (n_sub < 1 || n_sub > num_modes) return fock_set_error(FOCK_ERR_INVALID, "bad number of prepared modes");
  PrepArgs P;
  memset(&P, 0, sizeof(P));
  P.N = num_modes; P.D = cutoff; P.nsub = n_sub;
  for (int m = 0; m < num_modes; ++m) P.is_sub[m] = -1;
  for (int p = 0; p < n_sub; ++p) {
    if ((rc = check_mode(modes[p], num_modes, "mode"))) return rc;
    if (P.is_sub[modes[p]] >= 0) return fock_set_error(FOCK_ERR_INVALID, "The specified modes cannot appear multiple times.");
    P.is_sub[modes[p]] = p;
  }
  if (!sub || !in || !out || in == out) return fock_set_error(FOCK_ERR_INVALID, "bad buffers");
  if (n_sub < num_modes && !workspace) return fock_set_error(FOCK_ERR_INVALID, "workspace required");
  int64_t nred = 1, ntr = 1;
  for (int k = 0; k < 2 * (num_modes - n_sub); ++k) nred *= cutoff;
  for (int k = 0; k < n_sub; ++k) ntr *= cutoff;
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == FOCK_C64) {
    float2* red = (float2*)workspace;
    if (n_sub < num_modes) {
      partial_trace_kernel<float2><<<grid_for(nred, 256), 256, 0, st>>>((const float2*)in, red, nred, ntr, P);
      FOCK_LAUNCH_CHECK("partial_trace_kernel");
    } else {
      // the whole state is replaced: reduced state is the scalar trace
      partial_trace_kernel<float2><<<1, 32, 0, st>>>((const float2*)in, (float2*)workspace, 1, ntr, P);
      FOCK_LAUNCH_CHECK("partial_trace_kernel");
    }
    tensor_insert_kernel<float2><<<grid_for(n, 256), 256, 0, st>>>(red, (const double2*)sub, (float2*)out, n, P);
  } else {
    double2* red = (double2*)workspace;
    if (n_sub < num_modes)
      partial_trace_kernel<double2><<<grid_for(nred, 256), 256, 0, st>>>((const double2*)in, red, nred, ntr, P);
    else
      partial_trace_kernel<double2><<<1, 32, 0, st>>>((const double2*)in, red, 1, ntr, P);
    FOCK_LAUNCH_CHECK("partial_trace_kernel");
    tensor_insert_kernel<double2><<<grid_for(n, 256), 256, 0, st>>>(red, (const double2*)sub, (double2*)out, n, P);
  }
  FOCK_LAUNCH_CHECK("tensor_insert_kernel");
  return FOCK_OK;
}

// ---------------------------------------------------------------------------
// readouts
// ---------------------------------------------------------------------------
template <typename CT>
__global__ void probs_kernel(const CT* __restrict__ st, double* __restrict__ probs, int64_t n, int N, int D,
                             int pure) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (int64_t)gridDim.x * blockDim.x) {
    if (pure) {
      double2 x = to_d(st[idx]);
      probs[idx] = x.x * x.x + x.y * x.y;
    } else {
      int64_t t = idx, off = 0, w = 1;
      for (int m = N - 1; m >= 0; --m) {
        int d = (int)(t % D); t /= D;
        off += (int64_t)d * w * (D + 1);
        w *= (int64_t)D * D;
      }
      probs[idx] = to_d(st[off]).x;
    }
  }
}

extern "C" int fock_probs(int num_modes, int cutoff, int pure, int dtype, const void* state, double* probs,
                          void* stream) {
  int64_t n;
  int rc = check_state(num_modes, cutoff, 1, dtype, &n);
  if (rc) return rc;
  if ((rc = check_state(num_modes, cutoff, pure, dtype, nullptr))) return rc;
  if (!state || !probs) return fock_set_error(FOCK_ERR_INVALID, "null buffer");
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == FOCK_C64)
    probs_kernel<float2><<<grid_for(n, 256), 256, 0, st>>>((const float2*)state, probs, n, num_modes, cutoff, pure);
  else
    probs_kernel<double2><<<grid_for(n, 256), 256, 0, st>>>((const double2*)state, probs, n, num_modes, cutoff, pure);
  FOCK_LAUNCH_CHECK("probs_kernel");
  return FOCK_OK;
}

// marginal of one axis of a real (probability) or complex (|x|^2) tensor:
// per-CTA partial sums part[block][k]
__device__ __forceinline__ double weight_of(double x) { return x; }
__device__ __forceinline__ double weight_of(float2 x) { return (double)x.x * x.x + (double)x.y * x.y; }
__device__ __forceinline__ double weight_of(double2 x) { return x.x * x.x + x.y * x.y; }

template <typename T>
__global__ void marginal_kernel(const T* __restrict__ src, AxisView v, int D, double* __restrict__ part) {
  extern __shared__ double hist[];  // [D]
  for (int k = threadIdx.x; k < D; k += blockDim.x) hist[k] = 0.0;
  __syncthreads();
  // thread per column, one level at a time (keeps registers independent of D)
  for (int k = 0; k < D; ++k) {
    double acc = 0.0;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < v.ncols; j += (int64_t)gridDim.x * blockDim.x)
      acc += weight_of(src[col_base(v, j, D) + k * v.s1]);
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(&hist[k], acc);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < D; k += blockDim.x) part[(int64_t)blockIdx.x * D + k] = hist[k];
}

__global__ void sum_parts_kernel(const double* __restrict__ part, int nparts, int D, double* __restrict__ out) {
  int k = blockIdx.x;
  double a = 0.0;
  for (int p = threadIdx.x; p < nparts; p += 32) a += part[(int64_t)p * D + k];
  for (int off = 16; off > 0; off >>= 1) a += __shfl_xor_sync(0xffffffffu, a, off);
  if (threadIdx.x == 0) out[k] = a;
}

static int marginal_parts(int64_t ncols) {
  int64_t g = (ncols + 255) / 256;
  int64_t cap = (int64_t)fock_num_sms() * 4;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

extern "C" int64_t fock_marginals_workspace_bytes(int num_modes, int cutoff, int pure, int dtype) {
  (void)dtype;
  int64_t n = 1;
  for (int k = 0; k < num_modes; ++k) n *= cutoff;
  int64_t parts = (int64_t)fock_num_sms() * 4 * cutoff * 8;
  return parts + (pure ? 0 : n * 8) + 256;
}

extern "C" int fock_marginals(int num_modes, int cutoff, int pure, int dtype, const void* state, double* out,
                              void* workspace, void* stream) {
  int64_t n;
  int rc = check_state(num_modes, cutoff, pure, dtype, &n);
  if (rc) return rc;
  if (!state || !out || !workspace) return fock_set_error(FOCK_ERR_INVALID, "null buffer");
  cudaStream_t st = (cudaStream_t)stream;
  double* part = (double*)workspace;
  const int64_t part_bytes = (int64_t)fock_num_sms() * 4 * cutoff * 8;
  const double* probs = nullptr;
  if (!pure) {
    double* pr = (double*)((char*)workspace + ((part_bytes + 255) / 256) * 256);
    rc = fock_probs(num_modes, cutoff, 0, dtype, state, pr, stream);
    if (rc) return rc;
    probs = pr;
  }
  for (int m = 0; m < num_modes; ++m) {
    AxisView v = make_view1(num_modes, cutoff, m);
    const int g = marginal_parts(v.ncols);
    size_t sm = cutoff * sizeof(double);
    if (!pure) marginal_kernel<double><<<g, 256, sm, st>>>(probs, v, cutoff, part);
    else if (dtype == FOCK_C64) marginal_kernel<float2><<<g, 256, sm, st>>>((const float2*)state, v, cutoff, part);
    else marginal_kernel<double2><<<g, 256, sm, st>>>((const double2*)state, v, cutoff, part);
    FOCK_LAUNCH_CHECK("marginal_kernel");
    sum_parts_kernel<<<cutoff, 32, 0, st>>>(part, g, cutoff, out + (int64_t)m * cutoff);
    FOCK_LAUNCH_CHECK("sum_parts_kernel");
  }
  return FOCK_OK;
}

// reduced density matrix of one mode
template <typename CT>
__global__ void rdm_mixed_kernel(const CT* __restrict__ rho, int N, int D, int mode, int64_t ntr,
                                 double2* __restrict__ part) {
  // grid: (D*D entries, chunks)
  const int e = blockIdx.x;
  const int a = e / D, b = e - a * D;
  const int64_t chunk = (ntr + gridDim.y - 1) / gridDim.y;
  const int64_t t0 = blockIdx.y * chunk;
  int64_t t1 = t0 + chunk;
  if (t1 > ntr) t1 = ntr;
  double2 acc = make_double2(0.0, 0.0);
  for (int64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
    int64_t tt = t, off = 0, w = 1;
    for (int m = N - 1; m >= 0; --m) {
      int ka, kb;
      if (m == mode) { ka = a; kb = b; }
      else { ka = kb = (int)(tt % D); tt /= D; }
      off += kb * w; w *= D;
      off += ka * w; w *= D;
    }
    acc = cadd(acc, to_d(rho[off]));
  }
  __shared__ double2 red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = cadd(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(int64_t)blockIdx.y * D * D + e] = red[0];
}

__global__ void transpose_dm_kernel(const double2* __restrict__ c, double2* __restrict__ out, int D) {
  for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
    int a = e / D, b = e - a * D;
    out[a * D + b] = c[b * D + a];
  }
}

int launch_rdm_mixed(int dtype, const void* state, int num_modes, int D, int mode, int64_t ntr, int chunks,
                     double2* part, cudaStream_t st) {
  dim3 grid(D * D, chunks);
  if (dtype == FOCK_C64)
    rdm_mixed_kernel<float2><<<grid, 256, 0, st>>>((const float2*)state, num_modes, D, mode, ntr, part);
  else
    rdm_mixed_kernel<double2><<<grid, 256, 0, st>>>((const double2*)state, num_modes, D, mode, ntr, part);
  FOCK_LAUNCH_CHECK("rdm_mixed_kernel");
  return FOCK_OK;
}

int launch_transpose_dm(const double2* C, double2* out, int D, cudaStream_t st) {
  transpose_dm_kernel<<<1, 256, 0, st>>>(C, out, D);
  FOCK_LAUNCH_CHECK("transpose_dm_kernel");
  return FOCK_OK;
}

int check_reduced_dm1_args(int num_modes, int cutoff, int pure, int dtype, int mode, const void* state,
                           const void* out) {
  int64_t n;
  int rc = check_state(num_modes, cutoff, pure, dtype, &n);
  if (rc) return rc;
  if ((rc = check_mode(mode, num_modes, "mode"))) return rc;
  if (!state || !out) return fock_set_error(FOCK_ERR_INVALID, "null buffer");
  return FOCK_OK;
}

extern "C" int64_t fock_reduced_dm1_workspace_bytes(int num_modes, int cutoff, int pure, int dtype) {
  int64_t c = (int64_t)cutoff * cutoff;
  if (pure) {
    int64_t part = 0;
    for (int m = 0; m < num_modes; ++m) {
      AdjSched sc = make_adj_sched(dtype, make_view1(num_modes, cutoff, m), cutoff, LAYOUT_DENSE);
      if (sc.part_entries > part) part = sc.part_entries;
    }
    return (part + c) * 16 + 256;
  }
  return (64 + 1) * c * 16 + 256;
}

extern "C" int fock_reduced_dm1(int num_modes, int cutoff, int pure, int dtype, int mode, const void* state,
                                void* out, void* workspace, void* stream) {
  int64_t n;
  int rc = check_state(num_modes, cutoff, pure, dtype, &n);
  if (rc) return rc;
  if ((rc = check_mode(mode, num_modes, "mode"))) return rc;
  if (!state || !out || !workspace) return fock_set_error(FOCK_ERR_INVALID, "null buffer");
  cudaStream_t st = (cudaStream_t)stream;
  const int D = cutoff;
  double2* ws = (double2*)workspace;
  if (pure) {
    // C[u][v] = sum conj(psi[u]) psi[v] = rho[v][u]
    AxisView v = make_view1(num_modes, D, mode);
    const AdjSched sc = make_adj_sched(dtype, v, D, LAYOUT_DENSE);
    double2* C = ws;
    double2* cpart = ws + (int64_t)D * D;
    // the matrix is not needed (lam_in not written); pass any in-bounds pointer
    rc = launch_adjoint_partials(dtype, state, state, nullptr, v, D, LAYOUT_DENSE, C, 0, cpart, sc, st);
    if (rc) return rc;
    rc = launch_reduce_sched(cpart, sc, D, LAYOUT_DENSE, C, st);
    if (rc) return rc;
    transpose_dm_kernel<<<1, 256, 0, st>>>(C, (double2*)out, D);
    FOCK_LAUNCH_CHECK("transpose_dm_kernel");
    return FOCK_OK;
  }
  int64_t ntr = 1;
  for (int k = 0; k < num_modes - 1; ++k) ntr *= D;
  int chunks = (int)((ntr + 4095) / 4096);
  if (chunks > 64) chunks = 64;
  if (chunks < 1) chunks = 1;
  dim3 grid(D * D, chunks);
  if (dtype == FOCK_C64)
    rdm_mixed_kernel<float2><<<grid, 256, 0, st>>>((const float2*)state, num_modes, D, mode, ntr, ws);
  else
    rdm_mixed_kernel<double2><<<grid, 256, 0, st>>>((const double2*)state, num_modes, D, mode, ntr, ws);
  FOCK_LAUNCH_CHECK("rdm_mixed_kernel");
  rc = launch_reduce_partials(ws, chunks, (int64_t)D * D, (double2*)out, st);
  return rc;
}
