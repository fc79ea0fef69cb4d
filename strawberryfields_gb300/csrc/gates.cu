// FP64 gate-matrix builders on the device (rows G1-G5 of the hot path).
//
// Every matrix holds the exact matrix elements of the infinite-dimensional
// operator, truncated to the cutoff -- the convention of the builders the
// reference takes from thewalrus.fock_gradients (strawberryfields/backends/
// fockbackend/ops.py:219-343), pinned by the reference's analytic tests.
// The recurrences follow from the ladder-operator actions of each gate
// (strawberryfields/ops.py: Dgate :1497, Sgate :1612, BSgate :1864-1893,
// S2gate :2036-2066) and only ever step to lower indices, so truncation does
// not perturb the stored entries.  Derivatives with respect to r / theta are
// G*U with the gate generator G, evaluated on an extended-cutoff copy held in
// scratch (again exact after truncation); phase derivatives are index weights
// applied by the parameter-gradient kernel.
//
// One CTA builds one matrix; rows/blocks that depend on each other are
// separated by __syncthreads().
#include "gates.cuh"

#include <stdarg.h>
#include <stdio.h>
#include <string.h>

int gate_layout(int gate) {
  switch (gate) {
    case FOCK_ROTATION:
    case FOCK_KERR:
    case FOCK_DISPLACEMENT:
    case FOCK_SQUEEZE:
      return LAYOUT_DENSE;
    case FOCK_BEAMSPLITTER:
    case FOCK_MZGATE:
    case FOCK_CROSS_KERR:
      return LAYOUT_SUM;
    case FOCK_TWO_MODE_SQUEEZE:
    case FOCK_LOSS:
      return LAYOUT_DIFF;
    default:
      return 0;
  }
}

int64_t layout_entries(int layout, int D) {
  if (layout == LAYOUT_DENSE) return (int64_t)D * D;
  if (layout == LAYOUT_SUM || layout == LAYOUT_DIFF) return blk_total(D);
  return 0;
}

int64_t build_scratch_entries(int gate, int D) {
  switch (gate) {
    case FOCK_SQUEEZE: return (int64_t)(D + 2) * D;
    case FOCK_BEAMSPLITTER: return blk_total(D + 1);
    case FOCK_TWO_MODE_SQUEEZE: return blk_total(D + 1);
    case FOCK_MZGATE: {
      // full (untruncated) blocks N = 0..2D-2 of size N+1, three of them
      int64_t t = 0;
      for (int N = 0; N <= 2 * D - 2; ++N) t += (int64_t)(N + 1) * (N + 1);
      return 3 * t;
    }
    default: return 0;
  }
}

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 dmul(double2 a, double2 b) { return cmul(a, b); }
__device__ __forceinline__ double2 dscale(double2 a, double s) { return cscale(a, s); }
__device__ __forceinline__ double2 dexpi(double t) {
  double s, c;
  sincos(t, &s, &c);
  return make_double2(c, s);
}

// (out, in) coordinates of entry e of a layout
__device__ __forceinline__ void entry_coords(int layout, int D, int e, int& oa, int& ob, int& ia,
                                             int& ib, int& u, int& v, int& blk) {
  if (layout == LAYOUT_DENSE) {
    u = e / D;
    v = e - u * D;
    oa = u; ia = v; ob = 0; ib = 0; blk = 0;
    return;
  }
  // locate block
  int b = 0;
  int off = 0;
  int nb = 2 * D - 1;
  for (b = 0; b < nb; ++b) {
    int s = blk_size(D, b);
    if (e < off + s * s) break;
    off += s * s;
  }
  int s = blk_size(D, b);
  u = (e - off) / s;
  v = (e - off) - u * s;
  blk = b;
  int ks = (layout == LAYOUT_SUM);
  blk_coord(D, ks, b, u, oa, ob);
  blk_coord(D, ks, b, v, ia, ib);
}

__device__ __forceinline__ int dev_layout_entries(int layout, int D) {
  return layout == LAYOUT_DENSE ? D * D : blk_total(D);
}

// Per-CTA tables of a build.  The recurrences scale by sqrt(k) and 1/sqrt(k)
// of small integers, and the fused phases are exp(i angle) of index
// functions; FP64 square roots, divisions and sincos are long instruction
// sequences on GB300's FP64 pipe (1/64 of the FP32 rate), so each value is
// computed once per CTA instead of once per matrix entry.  The table entries
// are the same correctly rounded sqrt(k) and 1.0 / sqrt(k) the per-entry
// expressions gave.
#define BUILD_SQ_N (2 * FOCK_MAX_CUTOFF + 8)
#define BUILD_PH_D 24  // phase tables for cutoffs up to 24 (two D x D tables)
struct BuildTab {
  double sq[BUILD_SQ_N];
  double isq[BUILD_SQ_N];
  double2 ph[2][BUILD_PH_D * BUILD_PH_D];  // exp(i angle) of the input / output side
};

__device__ void build_tab_sqrt(BuildTab& T, int D) {
  const int n = min(2 * D + 8, BUILD_SQ_N);
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const double r = sqrt((double)k);
    T.sq[k] = r;
    T.isq[k] = k > 0 ? 1.0 / r : 0.0;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// builders (whole CTA); U -> M, dU/dp0 -> dM (may be null)
// ---------------------------------------------------------------------------

// Displacement: D[0,n] = e^{-r^2/2} (-conj(alpha))^n / sqrt(n!),
// sqrt(m+1) D[m+1,n] = sqrt(n) D[m,n-1] + alpha D[m,n];
// dD/dr[m,n] = e^{i phi} sqrt(m) D[m-1,n] - e^{-i phi} sqrt(n) D[m,n-1] - r D[m,n].
__device__ void build_displacement(double r, double phi, int D, double2* M, double2* dM, const BuildTab& T) {
  const double2 alpha = dscale(dexpi(phi), r);
  if (threadIdx.x == 0) {
    double2 v = make_double2(exp(-0.5 * r * r), 0.0);
    const double2 mac = make_double2(-alpha.x, alpha.y);  // -conj(alpha)
    M[0] = v;
    for (int n = 1; n < D; ++n) {
      v = dscale(dmul(v, mac), T.isq[n]);
      M[n] = v;
    }
  }
  __syncthreads();
  for (int m = 0; m < D - 1; ++m) {
    for (int n = threadIdx.x; n < D; n += blockDim.x) {
      double2 acc = dmul(alpha, M[m * D + n]);
      if (n > 0) acc = cadd(acc, dscale(M[m * D + n - 1], T.sq[n]));
      M[(m + 1) * D + n] = dscale(acc, T.isq[m + 1]);
    }
    __syncthreads();
  }
  if (dM) {
    const double2 e = dexpi(phi), ec = make_double2(e.x, -e.y);
    for (int idx = threadIdx.x; idx < D * D; idx += blockDim.x) {
      int m = idx / D, n = idx - m * D;
      double2 acc = dscale(M[idx], -r);
      if (m > 0) acc = cadd(acc, dmul(e, dscale(M[idx - D], T.sq[m])));
      if (n > 0) acc = csub(acc, dmul(ec, dscale(M[idx - 1], T.sq[n])));
      dM[idx] = acc;
    }
  }
  __syncthreads();
}

// Squeezing S(z) = exp((z* a^2 - z a^dag^2)/2): squeezed-vacuum column
// S[m,0] = -e^{i phi} tanh r sqrt((m-1)/m) S[m-2,0], S[0,0] = 1/sqrt(cosh r);
// S[m,n+1] = (sqrt(m) S[m-1,n] + e^{-i phi} sinh r sqrt(n) S[m,n-1]) / (cosh r sqrt(n+1)).
// Built on rows 0..D+1 (scratch X, row-major (D+2) x D) so that
// dS/dr = G S, G = (e^{-i phi} a^2 - e^{i phi} a^dag^2)/2, is exact.
__device__ void build_squeezing(double r, double phi, int D, double2* M, double2* dM, double2* X,
                                const BuildTab& T) {
  const int R = D + 2;
  const double c = cosh(r), s = sinh(r), t = tanh(r);
  const double2 e = dexpi(phi), ec = make_double2(e.x, -e.y);
  for (int i = threadIdx.x; i < R * D; i += blockDim.x) X[i] = make_double2(0.0, 0.0);
  __syncthreads();
  if (threadIdx.x == 0) {
    double2 v = make_double2(1.0 / sqrt(c), 0.0);
    X[0] = v;
    const double2 f = make_double2(-e.x * t, -e.y * t);
    for (int m = 2; m < R; m += 2) {
      v = dscale(dmul(f, v), sqrt((m - 1.0) / m));
      X[m * D] = v;
    }
  }
  __syncthreads();
  for (int n = 0; n < D - 1; ++n) {
    for (int m = threadIdx.x; m < R; m += blockDim.x) {
      double2 acc = make_double2(0.0, 0.0);
      if (m > 0) acc = dscale(X[(m - 1) * D + n], T.sq[m]);
      if (n > 0) acc = cadd(acc, dmul(ec, dscale(X[m * D + n - 1], s * T.sq[n])));
      X[m * D + n + 1] = dscale(acc, 1.0 / (c * T.sq[n + 1]));
    }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < D * D; idx += blockDim.x) {
    int m = idx / D, n = idx - m * D;
    M[idx] = X[m * D + n];
    if (dM) {
      double2 acc = dmul(ec, dscale(X[(m + 2) * D + n], 0.5 * sqrt((m + 1.0) * (m + 2.0))));
      if (m >= 2) acc = csub(acc, dmul(e, dscale(X[(m - 2) * D + n], 0.5 * sqrt(m * (m - 1.0)))));
      dM[idx] = acc;
    }
  }
  __syncthreads();
}

// Beamsplitter, photon-number-sum blocks at cutoff De = D+1 in scratch X.
// Entry E_N[i][k] = <i, N-i| B |k, N-k>:
//   i >= 1: sqrt(i) E_N[i][k] = t sqrt(k) E_{N-1}[i-1][k-1] - conj(rho) sqrt(N-k) E_{N-1}[i-1][k]
//   i == 0: sqrt(N) E_N[0][k] = t sqrt(N-k) E_{N-1}[0][k] + rho sqrt(k) E_{N-1}[0][k-1]
// (t = cos theta, rho = e^{i phi} sin theta; B^dag a1 B = t a1 - conj(rho) a2,
//  B^dag a2 B = t a2 + rho a1).  dB/dtheta = G B with
// G = e^{i phi} a1 a2^dag - e^{-i phi} a1^dag a2.
__device__ __forceinline__ double2 blk_get(const double2* X, int De, int ks, int N, int i, int k) {
  if (N < 0 || N > 2 * De - 2) return make_double2(0.0, 0.0);
  int lo = blk_lo(De, ks, N);
  int s = blk_size(De, N);
  int u = i - lo, v = k - lo;
  if (u < 0 || u >= s || v < 0 || v >= s) return make_double2(0.0, 0.0);
  return X[blk_offset(De, N) + u * s + v];
}

__device__ void build_beamsplitter_ext(double theta, double phi, int De, double2* X, const BuildTab& T) {
  const double t = cos(theta);
  const double2 rho = dscale(dexpi(phi), sin(theta));
  const double2 rhoc = make_double2(rho.x, -rho.y);
  if (threadIdx.x == 0) X[0] = make_double2(1.0, 0.0);
  __syncthreads();
  for (int N = 1; N <= 2 * De - 2; ++N) {
    const int s = blk_size(De, N), lo = blk_lo(De, 1, N), off = blk_offset(De, N);
    for (int e = threadIdx.x; e < s * s; e += blockDim.x) {
      int u = e / s, v = e - u * s;
      int i = lo + u, k = lo + v;
      double2 acc;
      if (i >= 1) {
        acc = dscale(blk_get(X, De, 1, N - 1, i - 1, k - 1), t * T.sq[k]);
        acc = csub(acc, dmul(rhoc, dscale(blk_get(X, De, 1, N - 1, i - 1, k), T.sq[N - k])));
        acc = dscale(acc, T.isq[i]);
      } else {
        acc = dscale(blk_get(X, De, 1, N - 1, 0, k), t * T.sq[N - k]);
        acc = cadd(acc, dmul(rho, dscale(blk_get(X, De, 1, N - 1, 0, k - 1), T.sq[k])));
        acc = dscale(acc, T.isq[N]);
      }
      X[off + e] = acc;
    }
    __syncthreads();
  }
}

// Two-mode squeezing S2 = exp(z a1^dag a2^dag - z* a1 a2), photon-number-
// difference blocks at cutoff De in scratch X.  Entry T_Delta[m][n] =
// <m, m-Delta| S2 |n, n-Delta>.  Base (first input of each block):
// T = lambda^u sqrt(C(u+|Delta|, |Delta|)) / cosh(r)^{|Delta|+1}, lambda = e^{i phi} tanh r,
// u the output position.  Recurrence (a1^dag S2 = S2 (c a1^dag + e^{-i phi} s a2)):
// T[m,n+1,p,q] = (sqrt(m) T[m-1,n,p,q] - e^{-i phi} s sqrt(q) T[m,n,p,q-1]) / (c sqrt(n+1)),
// processed in layers of the input's first coordinate.
// dT/dr = G T with G = e^{i phi} a1^dag a2^dag - e^{-i phi} a1 a2.
__device__ void build_s2_ext(double r, double phi, int De, double2* X, const BuildTab& T) {
  const double c = cosh(r), s = sinh(r), th = tanh(r);
  const double2 e = dexpi(phi), ec = make_double2(e.x, -e.y);
  const double2 lam = dscale(e, th);
  const int nb = 2 * De - 1;
  for (int L = 0; L < De; ++L) {
    // every (block, output position) whose input position v = L - lo lies in range
    for (int task = threadIdx.x; task < nb * De; task += blockDim.x) {
      int b = task / De, u = task - b * De;
      int sb = blk_size(De, b);
      if (u >= sb) continue;
      int lo = blk_lo(De, 0, b);
      int v = L - lo;
      if (v < 0 || v >= sb) continue;
      int delta = b - (De - 1);
      int ad = delta < 0 ? -delta : delta;
      double2 val;
      if (v == 0) {
        // lambda^u sqrt(C(u+ad, ad)) / c^{ad+1}
        double lg = 0.5 * (lgamma((double)(u + ad + 1)) - lgamma((double)(u + 1)) - lgamma((double)(ad + 1)));
        double mag = exp(lg) / pow(c, (double)(ad + 1));
        double2 lp = make_double2(1.0, 0.0);
        for (int k = 0; k < u; ++k) lp = dmul(lp, lam);
        val = dscale(lp, mag);
      } else {
        // target input (n+1, q) = (lo+v, lo+v-delta); output (m, p) = (lo+u, lo+u-delta)
        int m = lo + u;
        int n1 = lo + v;          // n + 1
        int q = lo + v - delta;
        // T[m-1, n, p, q]: block delta-1
        double2 t1 = make_double2(0.0, 0.0);
        if (m >= 1 && b >= 1) t1 = blk_get(X, De, 0, b - 1, m - 1, n1 - 1);
        // T[m, n, p, q-1]: same block, input position v-1
        double2 t2 = X[blk_offset(De, b) + u * sb + (v - 1)];
        double2 acc = dscale(t1, T.sq[m]);
        acc = csub(acc, dmul(ec, dscale(t2, s * T.sq[q])));
        val = dscale(acc, 1.0 / (c * T.sq[n1]));
      }
      X[blk_offset(De, b) + u * sb + v] = val;
    }
    __syncthreads();
  }
}

// copy the cutoff-D blocks out of cutoff-(D+1) storage and form G*U
// gen_kind 0: beamsplitter generator, 1: two-mode-squeeze generator
__device__ void blocks_truncate_and_derive(const double2* X, int D, int ks, double phi,
                                           int gen_kind, double2* M, double2* dM, const BuildTab& T) {
  const int De = D + 1;
  const double2 e = dexpi(phi), ec = make_double2(e.x, -e.y);
  const int tot = blk_total(D);
  for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
    int b = 0, off = 0;
    for (b = 0; b < 2 * D - 1; ++b) {
      int s = blk_size(D, b);
      if (idx < off + s * s) break;
      off += s * s;
    }
    int s = blk_size(D, b);
    int u = (idx - off) / s, v = (idx - off) - u * s;
    int oa, ob, ia, ib;
    blk_coord(D, ks, b, u, oa, ob);
    blk_coord(D, ks, b, v, ia, ib);
    // block index at the extended cutoff
    int be = ks ? b : (b + 1);  // DIFF: delta + De - 1 = (b - (D-1)) + D
    M[idx] = blk_get(X, De, ks, be, oa, ia);
    if (dM) {
      double2 acc;
      if (gen_kind == 0) {
        // e^{i phi} sqrt(m+1) sqrt(p) B[m+1, n, p-1, q] - e^{-i phi} sqrt(m) sqrt(p+1) B[m-1, n, p+1, q]
        acc = dmul(e, dscale(blk_get(X, De, 1, be, oa + 1, ia), T.sq[oa + 1] * T.sq[ob]));
        acc = csub(acc, dmul(ec, dscale(blk_get(X, De, 1, be, oa - 1, ia), T.sq[oa] * T.sq[ob + 1])));
      } else {
        // e^{i phi} sqrt(m) sqrt(p) T[m-1,n,p-1,q] - e^{-i phi} sqrt(m+1) sqrt(p+1) T[m+1,n,p+1,q]
        acc = dmul(e, dscale(blk_get(X, De, 0, be, oa - 1, ia), T.sq[oa] * T.sq[ob]));
        acc = csub(acc, dmul(ec, dscale(blk_get(X, De, 0, be, oa + 1, ia), T.sq[oa + 1] * T.sq[ob + 1])));
      }
      dM[idx] = acc;
    }
  }
  __syncthreads();
}

// Mach-Zehnder MZ(phi_in, phi_ex) = BS(pi/4,pi/2) (R(phi_in) x I) BS(pi/4,pi/2) (R(phi_ex) x I)
// (strawberryfields/ops.py:1951).  The external phase is carried as a fused
// input phase term by the caller; here M = B R_in B and dM/dphi_in =
// B (i n1 R_in) B on complete photon-number blocks (size N+1), then truncated.
__device__ void build_mzgate(double phi_in, int D, double2* M, double2* dM, double2* X, BuildTab& T) {
  // X: [full B blocks][B R_in][B i n1 R_in]
  // exp(i phi_in j), j < 2D - 1, in the CTA's phase table (2D - 1 <= BUILD_PH_D^2)
  double2* ph_in = T.ph[0];
  for (int j = threadIdx.x; j < 2 * D - 1; j += blockDim.x) ph_in[j] = dexpi(phi_in * j);
  int64_t tot = 0;
  for (int N = 0; N <= 2 * D - 2; ++N) tot += (int64_t)(N + 1) * (N + 1);
  double2* Bf = X;
  double2* T1 = X + tot;
  double2* T2 = X + 2 * tot;
  // full BS(pi/4, pi/2) blocks: <k', N-k'|B|k, N-k>, built column-free with the
  // same recurrence on untruncated blocks (cutoff 2D-1 is complete for N <= 2D-2)
  const double t = cos(0.25 * M_PI);
  const double2 rho = make_double2(0.0, sin(0.25 * M_PI));  // e^{i pi/2} sin(pi/4)
  const double2 rhoc = make_double2(0.0, -rho.y);
  int64_t off = 0, offp = 0;
  if (threadIdx.x == 0) Bf[0] = make_double2(1.0, 0.0);
  __syncthreads();
  for (int N = 1; N <= 2 * D - 2; ++N) {
    offp = off;
    off += (int64_t)N * N;
    const int s = N + 1, sp = N;
    for (int e = threadIdx.x; e < s * s; e += blockDim.x) {
      int i = e / s, k = e - i * s;
      double2 acc;
      auto prev = [&](int ii, int kk) -> double2 {
        if (ii < 0 || ii >= sp || kk < 0 || kk >= sp) return make_double2(0.0, 0.0);
        return Bf[offp + ii * sp + kk];
      };
      if (i >= 1) {
        acc = dscale(prev(i - 1, k - 1), t * T.sq[k]);
        acc = csub(acc, dmul(rhoc, dscale(prev(i - 1, k), T.sq[N - k])));
        acc = dscale(acc, T.isq[i]);
      } else {
        acc = dscale(prev(0, k), t * T.sq[N - k]);
        acc = cadd(acc, dmul(rho, dscale(prev(0, k - 1), T.sq[k])));
        acc = dscale(acc, T.isq[N]);
      }
      Bf[off + e] = acc;
    }
    __syncthreads();
  }
  // T1 = B R_in B, T2 = B (i k R_in) B per block
  off = 0;
  for (int N = 0; N <= 2 * D - 2; ++N) {
    const int s = N + 1;
    for (int e = threadIdx.x; e < s * s; e += blockDim.x) {
      int i = e / s, k = e - i * s;
      double2 a1 = make_double2(0.0, 0.0), a2 = make_double2(0.0, 0.0);
      for (int j = 0; j < s; ++j) {
        double2 x = dmul(dmul(Bf[off + i * s + j], ph_in[j]), Bf[off + j * s + k]);
        a1 = cadd(a1, x);
        a2 = cadd(a2, dscale(make_double2(-x.y, x.x), (double)j));
      }
      T1[off + e] = a1;
      T2[off + e] = a2;
    }
    off += (int64_t)s * s;
  }
  __syncthreads();
  // truncate into SUM blocks of cutoff D
  const int totD = blk_total(D);
  for (int idx = threadIdx.x; idx < totD; idx += blockDim.x) {
    int b = 0, o = 0;
    for (b = 0; b < 2 * D - 1; ++b) {
      int s = blk_size(D, b);
      if (idx < o + s * s) break;
      o += s * s;
    }
    int s = blk_size(D, b);
    int u = (idx - o) / s, v = (idx - o) - u * s;
    int lo = blk_lo(D, 1, b);
    int64_t fo = 0;
    for (int N = 0; N < b; ++N) fo += (int64_t)(N + 1) * (N + 1);
    int sf = b + 1;
    M[idx] = T1[fo + (lo + u) * sf + (lo + v)];
    if (dM) dM[idx] = T2[fo + (lo + u) * sf + (lo + v)];
  }
  __syncthreads();
}

// Loss superoperator on a (ket, bra) axis pair, difference blocks:
// N(T){|n><m|} = sum_l c(n,m,l) |n-l><m-l|,
// c = (1-T)^l T^{(n+m)/2 - l} / l! sqrt(n! m! / ((n-l)! (m-l)!))
// (strawberryfields/ops.py:1369-1376; Kraus form fockbackend/ops.py:471).
// dM = dc/dT = (-l (1-T)^(l-1) T^ex + ex (1-T)^l T^(ex-1)) * (the factorials)
// with ex = (n+m)/2 - l.
__device__ void build_loss(double T, int D, double2* M, double2* dM) {
  const int tot = blk_total(D);
  for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
    int oa, ob, ia, ib, u, v, b;
    entry_coords(LAYOUT_DIFF, D, idx, oa, ob, ia, ib, u, v, b);
    double val = 0.0, dval = 0.0;
    int l = ia - oa;
    if (l >= 0 && ib - ob == l) {
      int n = ia, m = ib;
      double lg = 0.5 * (lgamma(n + 1.0) + lgamma(m + 1.0) - lgamma(n - l + 1.0) - lgamma(m - l + 1.0)) -
                  lgamma(l + 1.0);
      double ex = 0.5 * (n + m) - l;
      const double f = exp(lg);
      val = pow(1.0 - T, (double)l) * pow(T, ex) * f;
      double d = 0.0;
      if (l > 0) d -= l * pow(1.0 - T, (double)(l - 1)) * pow(T, ex);
      if (ex > 0.0) d += ex * pow(1.0 - T, (double)l) * pow(T, ex - 1.0);
      dval = d * f;
    }
    M[idx] = make_double2(val, 0.0);
    if (dM) dM[idx] = make_double2(dval, 0.0);
  }
  __syncthreads();
}

__device__ void build_identity(int layout, int D, double2* M) {
  const int tot = dev_layout_entries(layout, D);
  for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
    int oa, ob, ia, ib, u, v, b;
    entry_coords(layout, D, idx, oa, ob, ia, ib, u, v, b);
    M[idx] = make_double2(u == v ? 1.0 : 0.0, 0.0);
  }
  __syncthreads();
}

// rotation / Kerr / cross-Kerr as their own (diagonal) matrices
__device__ void build_diag_gate(int gate, double p, int layout, int D, double2* M) {
  const int tot = dev_layout_entries(layout, D);
  for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
    int oa, ob, ia, ib, u, v, b;
    entry_coords(layout, D, idx, oa, ob, ia, ib, u, v, b);
    double2 val = make_double2(0.0, 0.0);
    if (u == v) {
      double ang = gate == FOCK_ROTATION ? p * oa : gate == FOCK_KERR ? p * (double)oa * oa : p * (double)oa * ob;
      val = dexpi(ang);
    }
    M[idx] = val;
  }
  __syncthreads();
}

__device__ void run_build_job(const BuildJob& J, const PhaseTerm* terms, const double* params,
                              double2* arena) {
  const double p0 = J.pidx >= 0 ? params[J.pidx] : J.v0;
  const double p1 = J.pidx >= 0 ? params[J.pidx + 1] : J.v1;
  double2* M = arena + J.m_off;
  double2* dM = J.dm_off >= 0 ? arena + J.dm_off : nullptr;
  double2* X = J.scratch_off >= 0 ? arena + J.scratch_off : nullptr;
  const int D = J.D;
  __shared__ BuildTab T;
  build_tab_sqrt(T, D);
  switch (J.gate) {
    case FOCK_DISPLACEMENT: build_displacement(p0, p1, D, M, dM, T); break;
    case FOCK_SQUEEZE: build_squeezing(p0, p1, D, M, dM, X, T); break;
    case FOCK_BEAMSPLITTER:
      build_beamsplitter_ext(p0, p1, D + 1, X, T);
      __syncthreads();
      blocks_truncate_and_derive(X, D, 1, p1, 0, M, dM, T);
      break;
    case FOCK_TWO_MODE_SQUEEZE:
      build_s2_ext(p0, p1, D + 1, X, T);
      __syncthreads();
      blocks_truncate_and_derive(X, D, 0, p1, 1, M, dM, T);
      break;
    case FOCK_MZGATE: build_mzgate(p0, D, M, dM, X, T); break;
    case FOCK_LOSS: build_loss(p0, D, M, dM); break;
    case FOCK_ROTATION:
    case FOCK_KERR:
    case FOCK_CROSS_KERR: build_diag_gate(J.gate, p0, J.layout, D, M); break;
    default: build_identity(J.layout, D, M); break;
  }
  // fused phases: M[e] *= exp(i sum_pre p f(in)) exp(i sum_post p f(out)),
  // from one table per side over the (a, b) coordinates (b = 0 for a dense
  // layout) -- one sincos per coordinate pair instead of one per entry
  if (J.nterm > 0 && D <= BUILD_PH_D) {
    int has_in = 0, has_out = 0;
    for (int k = 0; k < J.nterm; ++k) {
      if (terms[J.term0 + k].side) has_out = 1;
      else has_in = 1;
    }
    const int nbv = J.layout == LAYOUT_DENSE ? 1 : D;
    for (int i = threadIdx.x; i < 2 * D * nbv; i += blockDim.x) {
      const int side = i / (D * nbv), r = i - side * D * nbv;
      const int a = r / nbv, b = r - a * nbv;
      if (side ? !has_out : !has_in) continue;
      double ang = 0.0;
      for (int k = 0; k < J.nterm; ++k) {
        const PhaseTerm& P = terms[J.term0 + k];
        if (P.side != side) continue;
        double pv = P.pidx >= 0 ? params[P.pidx] : P.value;
        if (P.neg) pv = -pv;
        ang += pv * phase_fn(P.fn, a, b);
      }
      T.ph[side][a * D + b] = dexpi(ang);
    }
    __syncthreads();
    const int tot = dev_layout_entries(J.layout, D);
    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
      int oa, ob, ia, ib, u, v, b;
      entry_coords(J.layout, D, idx, oa, ob, ia, ib, u, v, b);
      double2 ph;
      if (has_out && has_in) ph = dmul(T.ph[1][oa * D + ob], T.ph[0][ia * D + ib]);
      else if (has_out) ph = T.ph[1][oa * D + ob];
      else ph = T.ph[0][ia * D + ib];
      M[idx] = dmul(M[idx], ph);
      if (dM) dM[idx] = dmul(dM[idx], ph);
    }
  } else if (J.nterm > 0) {
    const int tot = dev_layout_entries(J.layout, D);
    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
      int oa, ob, ia, ib, u, v, b;
      entry_coords(J.layout, D, idx, oa, ob, ia, ib, u, v, b);
      double ang = 0.0;
      for (int k = 0; k < J.nterm; ++k) {
        const PhaseTerm& P = terms[J.term0 + k];
        double pv = P.pidx >= 0 ? params[P.pidx] : P.value;
        if (P.neg) pv = -pv;
        ang += pv * (P.side ? phase_fn(P.fn, oa, ob) : phase_fn(P.fn, ia, ib));
      }
      double2 ph = dexpi(ang);
      M[idx] = dmul(M[idx], ph);
      if (dM) dM[idx] = dmul(dM[idx], ph);
    }
  }
  __syncthreads();
}

__global__ void build_jobs_kernel(const BuildJob* jobs, const PhaseTerm* terms, const double* params,
                                  double2* arena, int64_t param_stride, int64_t arena_stride) {
  // blockIdx.y: circuit of a batch (own parameters, own matrix arena)
  run_build_job(jobs[blockIdx.x], terms, params ? params + blockIdx.y * param_stride : nullptr,
                arena + blockIdx.y * arena_stride);
}

#define MAX_INLINE_TERMS 8
struct InlineBuild {
  BuildJob job;
  PhaseTerm terms[MAX_INLINE_TERMS];
};

__global__ void build_inline_kernel(InlineBuild b, double2* arena) {
  run_build_job(b.job, b.terms, nullptr, arena);
}

int launch_build_jobs(const BuildJob* d_jobs, int n_jobs, const PhaseTerm* d_terms,
                      const double* d_params, double2* arena, cudaStream_t st, int nb, int64_t param_stride,
                      int64_t arena_stride) {
  if (n_jobs <= 0) return FOCK_OK;
  build_jobs_kernel<<<dim3(n_jobs, nb), 256, 0, st>>>(d_jobs, d_terms, d_params, arena, param_stride,
                                                      arena_stride);
  FOCK_LAUNCH_CHECK("build_jobs_kernel");
  return FOCK_OK;
}

// Build one matrix with inline parameters (M at arena[0], dM after it, scratch after).
int build_single(int gate, int layout, int D, double p0, double p1, const PhaseTerm* terms,
                 int nterm, double2* M, double2* dM, double2* scratch, cudaStream_t st) {
  if (nterm > MAX_INLINE_TERMS) return fock_set_error(FOCK_ERR_INVALID, "too many phase terms");
  InlineBuild b;
  memset(&b, 0, sizeof(b));
  b.job.gate = gate;
  b.job.layout = layout;
  b.job.D = D;
  b.job.pidx = -1;
  b.job.v0 = p0;
  b.job.v1 = p1;
  b.job.term0 = 0;
  b.job.nterm = nterm;
  // offsets relative to M
  b.job.m_off = 0;
  b.job.dm_off = dM ? (int64_t)(dM - M) : -1;
  b.job.scratch_off = scratch ? (int64_t)(scratch - M) : -1;
  for (int k = 0; k < nterm; ++k) b.terms[k] = terms[k];
  build_inline_kernel<<<1, 256, 0, st>>>(b, M);
  FOCK_LAUNCH_CHECK("build_inline_kernel");
  return FOCK_OK;
}

// ---------------------------------------------------------------------------
// parameter gradients: grads[p] = sum over contributions of
// Re sum_e C[e] * X[e], X = dM or M * i * scale * weight
// ---------------------------------------------------------------------------
__global__ void param_grads_kernel(const GradOp* ops, const GradContrib* contrib, const int* pstart,
                                   const int* plist, const double2* arena, const double2* carena,
                                   double* grads, int n_params, int64_t arena_stride, int64_t carena_stride) {
  const int p = blockIdx.x;
  // blockIdx.y: circuit of a batch
  arena += blockIdx.y * arena_stride;
  carena += blockIdx.y * carena_stride;
  grads += (int64_t)blockIdx.y * n_params;
  __shared__ double red[256];
  double total = 0.0;
  for (int q = pstart[p]; q < pstart[p + 1]; ++q) {
    const GradContrib G = contrib[plist[q]];
    const GradOp O = ops[G.op];
    const double2* M = arena + O.m_off;
    const double2* dM = O.dm_off >= 0 ? arena + O.dm_off : nullptr;
    const double2* C = carena + O.c_off;
    double acc = 0.0;
    for (int e = threadIdx.x; e < O.nent; e += blockDim.x) {
      double2 x;
      if (G.type == GC_DM) {
        x = dM ? dM[e] : make_double2(0.0, 0.0);
      } else {
        int oa, ob, ia, ib, u, v, b;
        entry_coords(O.layout, O.D, e, oa, ob, ia, ib, u, v, b);
        double w;
        if (G.type == GC_W_IN) w = phase_fn(G.fn, ia, ib);
        else if (G.type == GC_W_OUT) w = phase_fn(G.fn, oa, ob);
        else w = phase_fn(G.fn, oa, ob) - phase_fn(G.fn, ia, ib);
        w *= G.scale;
        double2 m = M[e];
        x = make_double2(-m.y * w, m.x * w);  // i w M
      }
      double2 c = C[e];
      if (O.conj) c.y = -c.y;        // Re(C conj(dM)) = Re(conj(C) dM) for a conj(M) op
      acc += c.x * x.x - c.y * x.y;  // Re(c x)
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) total += red[0];
    __syncthreads();
  }
  if (threadIdx.x == 0) grads[p] = total;
}

int launch_param_grads(const GradOp* d_ops, const GradContrib* d_contrib, const int* d_pstart,
                       const int* d_plist, int n_params, const PhaseTerm* d_terms,
                       const double2* arena, const double2* carena, double* grads,
                       cudaStream_t st, int nb, int64_t arena_stride, int64_t carena_stride) {
  (void)d_terms;
  if (n_params <= 0) return FOCK_OK;
  param_grads_kernel<<<dim3(n_params, nb), 256, 0, st>>>(d_ops, d_contrib, d_pstart, d_plist, arena, carena,
                                                         grads, n_params, arena_stride, carena_stride);
  FOCK_LAUNCH_CHECK("param_grads_kernel");
  return FOCK_OK;
}

// ---------------------------------------------------------------------------
// C ABI: single-gate matrices
// ---------------------------------------------------------------------------
extern "C" int64_t fock_gate_matrix_entries(int kind, int cutoff) {
  if (cutoff < 1 || cutoff > FOCK_MAX_CUTOFF) return 0;
  return layout_entries(gate_layout(kind), cutoff);
}

extern "C" int64_t fock_gate_workspace_bytes(int kind, int cutoff) {
  if (cutoff < 1 || cutoff > FOCK_MAX_CUTOFF || gate_layout(kind) == 0) return 0;
  int64_t n = 2 * layout_entries(gate_layout(kind), cutoff) + build_scratch_entries(kind, cutoff);
  return n * (int64_t)sizeof(double2) + 256;
}

extern "C" int fock_gate_matrix(int kind, double p0, double p1, int cutoff, void* out, void* dout,
                                void* workspace, void* stream) {
  const int layout = gate_layout(kind);
  if (layout == 0) return fock_set_error(FOCK_ERR_INVALID, "unknown gate kind %d", kind);
  if (cutoff < 1 || cutoff > FOCK_MAX_CUTOFF)
    return fock_set_error(FOCK_ERR_INVALID, "cutoff must be in [1, %d], got %d", FOCK_MAX_CUTOFF, cutoff);
  if (!out) return fock_set_error(FOCK_ERR_INVALID, "null output pointer");
  const int64_t ns = build_scratch_entries(kind, cutoff);
  if (ns > 0 && !workspace) return fock_set_error(FOCK_ERR_INVALID, "workspace required for this gate");
  cudaStream_t st = (cudaStream_t)stream;
  // The builder addresses dM and scratch relative to M, so stage everything in
  // the workspace when the caller's buffers are separate.
  const int64_t ne = layout_entries(layout, cutoff);
  double2* ws = (double2*)workspace;
  // MZ(phi_in, phi_ex): the external phase R(phi_ex) on mode 1 acts first
  PhaseTerm mz_ex = {FN_A, 0, -1, 0, p1};
  const int nt = kind == FOCK_MZGATE ? 1 : 0;
  if (ws) {
    double2* M = ws;
    double2* dM = dout ? ws + ne : nullptr;
    double2* X = ns > 0 ? ws + 2 * ne : nullptr;
    int rc = build_single(kind, layout, cutoff, p0, p1, &mz_ex, nt, M, dM, X, st);
    if (rc) return rc;
    FOCK_CUDA_TRY(cudaMemcpyAsync(out, M, ne * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    if (dout) FOCK_CUDA_TRY(cudaMemcpyAsync(dout, dM, ne * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    return FOCK_OK;
  }
  // no scratch needed and no workspace: build in place (dout must follow out)
  if (dout) return fock_set_error(FOCK_ERR_INVALID, "derivatives need a workspace");
  return build_single(kind, layout, cutoff, p0, p1, &mz_ex, nt, (double2*)out, nullptr, nullptr, st);
}

__global__ void expand_blocks_kernel(int ks, int D, const double2* blocks, double2* dense) {
  const int tot = blk_total(D);
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < tot; idx += gridDim.x * blockDim.x) {
    int oa, ob, ia, ib, u, v, b;
    entry_coords(ks ? LAYOUT_SUM : LAYOUT_DIFF, D, idx, oa, ob, ia, ib, u, v, b);
    // dense [out1][in1][out2][in2]
    int64_t o = (((int64_t)oa * D + ia) * D + ob) * D + ib;
    dense[o] = blocks[idx];
  }
}

extern "C" int fock_expand_blocks(int kind, int cutoff, const void* blocks, void* dense, void* stream) {
  const int layout = gate_layout(kind);
  if (layout != LAYOUT_SUM && layout != LAYOUT_DIFF)
    return fock_set_error(FOCK_ERR_INVALID, "gate kind %d is not a two-axis block gate", kind);
  if (cutoff < 1 || cutoff > FOCK_MAX_CUTOFF) return fock_set_error(FOCK_ERR_INVALID, "bad cutoff");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t D4 = (int64_t)cutoff * cutoff * cutoff * cutoff;
  FOCK_CUDA_TRY(cudaMemsetAsync(dense, 0, D4 * sizeof(double2), st));
  expand_blocks_kernel<<<64, 256, 0, st>>>(layout == LAYOUT_SUM, cutoff, (const double2*)blocks,
                                           (double2*)dense);
  FOCK_LAUNCH_CHECK("expand_blocks_kernel");
  return FOCK_OK;
}
