// Phase-space readouts of a one-mode density matrix.
//
// Wigner function on a grid -- BaseFockState.wigner of the reference
// (strawberryfields/backends/states.py:730-785), which sums
// rho[m][n] W_{|m><n|}(x, p) over a table of D complex grids filled by a
// two-index recurrence.  Here one thread evaluates one grid point with no
// table: the same sum is ordered by diagonal k = n - m and each diagonal's
// terms come from the Laguerre form of W_{|m><m+k|},
//
//   W_{|m><m+k|}(A) = e^{-2|A|^2}/pi * (2A)^k / sqrt(k!)
//                     * (-1)^m sqrt(m! k! / (m+k)!) L_m^k(4|A|^2),
//   A = (x + i p) / sqrt(2 hbar),
//
// (Cahill and Glauber, Phys. Rev. 177, 1882 (1969)), with the normalised
// Laguerre values F_m = (-1)^m sqrt(m! k!/(m+k)!) L_m^k(y) from the
// three-term recurrence in m
//
//   F_0 = 1,  F_{m+1} = -[(2m+1+k-y) F_m + sqrt(m(m+k)) F_{m-1}] / sqrt((m+1)(m+1+k)).
//
// W = (1/hbar) * sum_k w_k Re[(e^{-y/2}/pi) (2A)^k/sqrt(k!) * sum_m rho[m][m+k] F_m],
// w_0 = 1, w_k = 2 (the k < 0 diagonals are the complex conjugates).  All in
// FP64; the recurrence constants and the matrix diagonals are staged in
// shared memory once per CTA.
#include "fock_common.cuh"

#include <math.h>

#include <algorithm>

namespace {

constexpr int WIG_THREADS = 256;

__global__ void __launch_bounds__(WIG_THREADS)
    wigner_kernel(const double2* __restrict__ rho, int D, const double* __restrict__ xvec, int nx,
                  const double* __restrict__ pvec, int np, double scale, double inv_hbar, double* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  // diag[k][m] = rho[m][m+k]; up[k][m] = 1/sqrt((m+1)(m+1+k)); dn[k][m] = sqrt(m(m+k));
  // hk[k] = 2/sqrt(k+1)
  double2* diag = reinterpret_cast<double2*>(smem);
  double* up = reinterpret_cast<double*>(diag + D * D);
  double* dn = up + D * D;
  double* hk = dn + D * D;
  for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
    const int k = e / D, m = e - k * D;
    diag[e] = m + k < D ? rho[m * D + m + k] : make_double2(0.0, 0.0);
    up[e] = 1.0 / sqrt((double)(m + 1) * (double)(m + 1 + k));
    dn[e] = sqrt((double)m * (double)(m + k));
  }
  for (int k = threadIdx.x; k < D; k += blockDim.x) hk[k] = 2.0 / sqrt((double)(k + 1));
  __syncthreads();
  const int64_t n = (int64_t)nx * np;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n; idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / nx;  // p index (row)
    const int64_t j = idx - i * nx;
    const double ar = xvec[j] * scale, ai = pvec[i] * scale;
    const double y = 4.0 * (ar * ar + ai * ai);
    double hr = exp(-0.5 * y) * (1.0 / M_PI), hi = 0.0;
    double W = 0.0;
    for (int k = 0; k < D; ++k) {
      const double2* dk = diag + k * D;
      const double* uk = up + k * D;
      const double* vk = dn + k * D;
      double sr = 0.0, si = 0.0, f = 1.0, fm = 0.0;
      const int mmax = D - k;
      for (int m = 0; m < mmax; ++m) {
        const double2 r = dk[m];
        sr = fma(r.x, f, sr);
        si = fma(r.y, f, si);
        const double fn = -fma(2.0 * m + 1.0 + k - y, f, vk[m] * fm) * uk[m];
        fm = f;
        f = fn;
      }
      const double t = hr * sr - hi * si;
      W += k == 0 ? t : 2.0 * t;
      const double c = hk[k];
      const double nr = c * (hr * ar - hi * ai);
      const double ni = c * (hr * ai + hi * ar);
      hr = nr;
      hi = ni;
    }
    out[idx] = W * inv_hbar;
  }
}

}  // namespace

extern "C" int fock_wigner(int cutoff, const void* rho, const double* xvec, int nx, const double* pvec, int np,
                           double hbar, double* out, void* stream) {
  if (cutoff < 1 || cutoff > FOCK_MAX_CUTOFF) return fock_set_error(FOCK_ERR_INVALID, "cutoff out of range");
  if (nx < 0 || np < 0) return fock_set_error(FOCK_ERR_INVALID, "negative grid size");
  if (!(hbar > 0.0)) return fock_set_error(FOCK_ERR_INVALID, "hbar must be positive");
  if ((int64_t)nx * np == 0) return FOCK_OK;
  if (!rho || !xvec || !pvec || !out) return fock_set_error(FOCK_ERR_INVALID, "null pointer");
  const int D = cutoff;
  const size_t smem = (size_t)D * D * (sizeof(double2) + 2 * sizeof(double)) + D * sizeof(double);
  if (smem > 48 * 1024)
    FOCK_CUDA_TRY(cudaFuncSetAttribute(wigner_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t n = (int64_t)nx * np;
  const int64_t want = (n + WIG_THREADS - 1) / WIG_THREADS;
  const int grid = (int)std::min<int64_t>(want, (int64_t)fock_num_sms() * 8);
  wigner_kernel<<<grid, WIG_THREADS, smem, (cudaStream_t)stream>>>(
      (const double2*)rho, D, xvec, nx, pvec, np, 1.0 / sqrt(2.0 * hbar), 1.0 / hbar, out);
  FOCK_CUDA_TRY(cudaGetLastError());
  return FOCK_OK;
}
