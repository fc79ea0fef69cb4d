// General N-mode Gaussian gate (Ggate): its Fock matrix from the
// multidimensional Hermite recurrence, and a dense apply on k modes.
//
// The reference builds the gate in its TF backend
// (strawberryfields/backends/tfbackend/ops.py:457-572): `choi_trick` maps the
// symplectic matrix S and displacement d to (R, y, C) -- done on the host
// here, in FP64 -- and thewalrus's renormalised multidimensional Hermite
// polynomials give G[k] = C H_k^R(y) / sqrt(k!) for the multi-index
// k = (out_1..out_m, in_1..in_m).  The renormalised recurrence
//
//   G[k] = (y_i G[k - e_i] - sum_j R_ij sqrt(k_j - delta_ij) G[k - e_i - e_j]) / sqrt(k_i),
//
// i the first nonzero index of k, reads only entries whose index i is one
// smaller and whose earlier indices are zero.  So the entries with
// k_0..k_{i-1} = 0 and k_i = v form a slab that depends only on the slab
// k_i = v - 1: one launch per (i, v), last index first, every entry of a
// slab in parallel (n (D - 1) launches, n = 2m).
//
// The apply gathers the D^k amplitudes of one column (the gate's axes in
// gate order; all other axes fixed) into shared memory and forms
// out[o] = sum_i G[o][i] x[i] with the matrix stored transposed in the state
// precision (consecutive threads read consecutive o).  A density matrix takes
// G on the ket axes and conj(G) on the bra axes (two passes).
#include "fock_common.cuh"

#include <string.h>

#include <algorithm>

namespace {

constexpr int GG_MAX_N = 6;  // 2m indices: up to three modes
constexpr int GG_THREADS = 256;
constexpr int GG_MAX_FIBER = 4096;

struct HermArgs {
  int n, D;
  double2 R[GG_MAX_N * GG_MAX_N];
  double2 y[GG_MAX_N];
  double2 C;
};

__global__ void hermite_origin_kernel(double2* G, HermArgs a) { G[0] = a.C; }

// slab (i, v): entries k = (0,..,0, v, t) with t over the trailing n-1-i indices
__global__ void hermite_slab_kernel(double2* __restrict__ G, const __grid_constant__ HermArgs a, int i, int v,
                                    int64_t slab) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= slab) return;
  const int n = a.n, D = a.D;
  // strides of the C-order multi-index
  int64_t stride[GG_MAX_N];
  int64_t s = 1;
  for (int j = n - 1; j >= 0; --j) {
    stride[j] = s;
    s *= D;
  }
  const int64_t idx = (int64_t)v * stride[i] + t;
  const int64_t km = idx - stride[i];  // k - e_i
  double2 acc = cmul(a.y[i], G[km]);
  // trailing indices of k - e_i (k_j for j > i; index i itself is v - 1)
  int64_t rem = t;
  for (int j = n - 1; j >= i; --j) {
    int kj;
    if (j == i) {
      kj = v - 1;
    } else {
      kj = (int)(rem % D);
      rem /= D;
    }
    if (kj > 0) {
      const double2 g = G[km - stride[j]];
      const double sq = sqrt((double)kj);
      const double2 r = a.R[i * n + j];
      acc.x -= sq * (r.x * g.x - r.y * g.y);
      acc.y -= sq * (r.x * g.y + r.y * g.x);
    }
  }
  const double inv = 1.0 / sqrt((double)v);
  G[idx] = make_double2(acc.x * inv, acc.y * inv);
}

// GT[i][o] = M[o][i] (conj with cj) in the state precision; M rows are the
// output multi-index of the k gate modes, columns the input one
template <typename CT>
__global__ void gg_transpose_kernel(const double2* __restrict__ M, CT* __restrict__ GT, int F, int cj) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)F * F) return;
  const int64_t o = e / F, i = e - o * F;
  double2 m = M[e];
  if (cj) m.y = -m.y;
  GT[i * F + o] = to_c(m, (CT*)nullptr);
}

struct ModesView {
  int naxes, D, k;
  int ax[GG_MAX_N];             // state axis of gate mode j (gate order)
  int64_t stride[FOCK_MAX_AXES];  // element stride of each state axis
  int rest_ax[FOCK_MAX_AXES];   // the other axes, slowest first
  int nrest;
  int64_t ncols, F;
};

template <typename CT>
__global__ void __launch_bounds__(GG_THREADS)
    gg_apply_kernel(const CT* __restrict__ in, CT* __restrict__ out, const CT* __restrict__ GT,
                    const __grid_constant__ ModesView mv) {
  extern __shared__ __align__(16) unsigned char smem[];
  CT* x = reinterpret_cast<CT*>(smem);
  int64_t* off = reinterpret_cast<int64_t*>(smem + ((mv.F * sizeof(CT) + 15) & ~(size_t)15));
  const int F = (int)mv.F;
  // fiber offsets: gate multi-index (C order over the k gate modes) -> element offset
  for (int f = threadIdx.x; f < F; f += blockDim.x) {
    int64_t o = 0, r = f;
    for (int j = mv.k - 1; j >= 0; --j) {
      o += (r % mv.D) * mv.stride[mv.ax[j]];
      r /= mv.D;
    }
    off[f] = o;
  }
  for (int64_t col = blockIdx.x; col < mv.ncols; col += gridDim.x) {
    int64_t base = 0, r = col;
    for (int j = mv.nrest - 1; j >= 0; --j) {
      base += (r % mv.D) * mv.stride[mv.rest_ax[j]];
      r /= mv.D;
    }
    __syncthreads();  // offsets ready; the previous column's x is consumed
    for (int f = threadIdx.x; f < F; f += blockDim.x) x[f] = in[base + off[f]];
    __syncthreads();
    for (int o = threadIdx.x; o < F; o += blockDim.x) {
      CT acc = czero<CT>();
      for (int i = 0; i < F; ++i) cfma(acc, GT[(int64_t)i * F + o], x[i]);
      out[base + off[o]] = acc;
    }
  }
}

int make_modes_view(int naxes, int D, int k, const int* axes, ModesView* mv) {
  memset(mv, 0, sizeof(*mv));
  mv->naxes = naxes;
  mv->D = D;
  mv->k = k;
  int64_t s = 1;
  for (int a = naxes - 1; a >= 0; --a) {
    mv->stride[a] = s;
    s *= D;
  }
  bool used[FOCK_MAX_AXES] = {false};
  mv->F = 1;
  for (int j = 0; j < k; ++j) {
    if (axes[j] < 0 || axes[j] >= naxes || used[axes[j]]) return fock_set_error(FOCK_ERR_INVALID, "bad gate modes");
    used[axes[j]] = true;
    mv->ax[j] = axes[j];
    mv->F *= D;
  }
  mv->ncols = 1;
  for (int a = 0; a < naxes; ++a)
    if (!used[a]) {
      mv->rest_ax[mv->nrest++] = a;
      mv->ncols *= D;
    }
  if (mv->F > GG_MAX_FIBER) return fock_set_error(FOCK_ERR_UNSUPPORTED, "gate on %d modes of cutoff %d: %lld amplitudes per column (max %d)", k, D, (long long)mv->F, GG_MAX_FIBER);
  return FOCK_OK;
}

template <typename CT>
int gg_apply_t(const double2* M, const ModesView& mv, const void* in, void* out, void* work, int cj,
               cudaStream_t st) {
  CT* GT = reinterpret_cast<CT*>(work);
  const int64_t FF = mv.F * mv.F;
  gg_transpose_kernel<CT><<<(unsigned)((FF + 255) / 256), 256, 0, st>>>(M, GT, (int)mv.F, cj);
  FOCK_CUDA_TRY(cudaGetLastError());
  const size_t sm = ((mv.F * sizeof(CT) + 15) & ~(size_t)15) + mv.F * sizeof(int64_t);
  if (sm > 48 * 1024)
    FOCK_CUDA_TRY(cudaFuncSetAttribute(gg_apply_kernel<CT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  const int grid = (int)std::min<int64_t>(mv.ncols, (int64_t)fock_num_sms() * 8);
  gg_apply_kernel<CT><<<grid, GG_THREADS, sm, st>>>((const CT*)in, (CT*)out, GT, mv);
  FOCK_CUDA_TRY(cudaGetLastError());
  return FOCK_OK;
}

}  // namespace

extern "C" int fock_gaussian_gate_matrix(int num_gate_modes, int cutoff, const double* R, const double* y,
                                         const double* C, void* mat, void* stream) {
  const int m = num_gate_modes, D = cutoff;
  if (m < 1 || 2 * m > GG_MAX_N) return fock_set_error(FOCK_ERR_UNSUPPORTED, "Gaussian gate on %d modes (1..3)", m);
  if (D < 1 || D > FOCK_MAX_CUTOFF) return fock_set_error(FOCK_ERR_INVALID, "cutoff out of range");
  if (!R || !y || !C || !mat) return fock_set_error(FOCK_ERR_INVALID, "null pointer");
  HermArgs a;
  memset(&a, 0, sizeof(a));
  a.n = 2 * m;
  a.D = D;
  for (int e = 0; e < a.n * a.n; ++e) a.R[e] = make_double2(R[2 * e], R[2 * e + 1]);
  for (int e = 0; e < a.n; ++e) a.y[e] = make_double2(y[2 * e], y[2 * e + 1]);
  a.C = make_double2(C[0], C[1]);
  double2* G = (double2*)mat;
  cudaStream_t st = (cudaStream_t)stream;
  hermite_origin_kernel<<<1, 1, 0, st>>>(G, a);
  FOCK_CUDA_TRY(cudaGetLastError());
  for (int i = a.n - 1; i >= 0; --i) {
    int64_t slab = 1;
    for (int j = i + 1; j < a.n; ++j) slab *= D;
    for (int v = 1; v < D; ++v) {
      hermite_slab_kernel<<<(unsigned)((slab + 255) / 256), 256, 0, st>>>(G, a, i, v, slab);
      FOCK_CUDA_TRY(cudaGetLastError());
    }
  }
  return FOCK_OK;
}

extern "C" int64_t fock_apply_modes_workspace_bytes(int k, int cutoff, int dtype) {
  int64_t F = 1;
  for (int j = 0; j < k; ++j) F *= cutoff;
  return F * F * (dtype == FOCK_C64 ? 8 : 16);
}

extern "C" int fock_apply_modes(int num_modes, int cutoff, int pure, int dtype, int k, const int* modes,
                                const void* mat, const void* in, void* out, void* tmp, void* workspace,
                                void* stream) {
  if (num_modes < 1 || cutoff < 1 || cutoff > FOCK_MAX_CUTOFF || (pure ? num_modes : 2 * num_modes) > FOCK_MAX_AXES)
    return fock_set_error(FOCK_ERR_INVALID, "bad state shape");
  if (dtype != FOCK_C64 && dtype != FOCK_C128) return fock_set_error(FOCK_ERR_INVALID, "bad dtype");
  if (k < 1 || k > num_modes || !modes) return fock_set_error(FOCK_ERR_INVALID, "bad gate modes");
  if (!mat || !in || !out || in == out || !workspace) return fock_set_error(FOCK_ERR_INVALID, "bad buffers");
  cudaStream_t st = (cudaStream_t)stream;
  const int naxes = pure ? num_modes : 2 * num_modes;
  int axes[GG_MAX_N];
  if (k > GG_MAX_N) return fock_set_error(FOCK_ERR_UNSUPPORTED, "gate on %d modes", k);
  for (int j = 0; j < k; ++j) {
    if (modes[j] < 0 || modes[j] >= num_modes) return fock_set_error(FOCK_ERR_INVALID, "mode %d out of range", modes[j]);
    axes[j] = pure ? modes[j] : 2 * modes[j];
  }
  ModesView mv;
  int rc = make_modes_view(naxes, cutoff, k, axes, &mv);
  if (rc) return rc;
  auto run = [&](const ModesView& v, const void* src, void* dst, int cj) {
    return dtype == FOCK_C64 ? gg_apply_t<float2>((const double2*)mat, v, src, dst, workspace, cj, st)
                             : gg_apply_t<double2>((const double2*)mat, v, src, dst, workspace, cj, st);
  };
  if (pure) return run(mv, in, out, 0);
  if (!tmp || tmp == in || tmp == out) return fock_set_error(FOCK_ERR_INVALID, "mixed states need a temporary state buffer");
  if ((rc = run(mv, in, tmp, 0))) return rc;
  for (int j = 0; j < k; ++j) axes[j] = 2 * modes[j] + 1;
  ModesView mb;
  if ((rc = make_modes_view(naxes, cutoff, k, axes, &mb))) return rc;
  return run(mb, tmp, out, 1);
}
