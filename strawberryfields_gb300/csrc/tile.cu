// Fused op groups on a three-mode tile held in shared memory (pure states,
// complex64).
//
// A state small enough to stay in L2 (the 6-mode cutoff-12 ket is 24 MB)
// spends most of a one-op launch in ramp-up, tail and latency, not in moving
// bytes.  Consecutive ops whose modes all lie in one set of three modes
// {t0 < t1 < t2} form a group: the state is then a set of independent
// columns (the indices of the other modes), each holding a D^3 tile, and one
// launch applies every op of the group to the tiles it holds in shared memory
// -- the state crosses L2 once per group instead of once per op.
//
// Forward: a CTA takes TC consecutive columns, copies their tiles into shared
// memory (lanes over columns when the innermost mode is not in the tile,
// else over the tile's contiguous innermost axis), and for each op stages the
// op's matrix (FP64 -> complex64) and applies it to every fibre of the tile:
// a dense D x D matrix along one tile axis, or the photon-number blocks of a
// two-mode op along a pair of tile axes (the selection rules of
// strawberryfields/backends/fockbackend/circuit.py:219-365).  Each op's output
// is written where the sweep stores it (every op's output when the adjoint
// needs them all), so the stored states are those of the per-op sweep.
//
// Adjoint: a CTA holds lam (the adjoint of the group's output) for its
// columns and walks the group's ops in reverse: it loads the op's stored
// input tile, forms this CTA's partial C = sum conj(lam_out) psi_in^T of the
// op (C entries dealt to the threads, fibres split into G groups when the
// entries are few) and writes it to the op's partial-sum region, then
// applies M^dagger to lam in place.  The partials are reduced by the plan's
// fixed-order reduction after the sweep (plane layout: entry e of CTA x at
// x * nent + e).
#include "apply.cuh"

#include <string.h>

#include <algorithm>

namespace {

constexpr int kTlThreads = TL_THREADS;

// tile-element stride of tile axis a (0: slowest)
__device__ __forceinline__ int tl_es(int D, int a) { return a == 0 ? D * D : (a == 1 ? D : 1); }

// photon-number block b of a two-mode op on tile axes (ta < tb): first
// element and step in tile-element units, and the block's size
__device__ __forceinline__ void tl_block(int D, int layout, int b, int esa, int esb, int& base, int& step, int& s) {
  s = blk_size(D, b);
  if (layout == LAYOUT_SUM) {
    const int lo = blk_lo(D, 1, b);
    base = lo * esa + (b - lo) * esb;
    step = esa - esb;
  } else {
    const int delta = b - (D - 1);
    const int lo = delta > 0 ? delta : 0;
    base = lo * esa + (lo - delta) * esb;
    step = esa + esb;
  }
}

// Stage op's matrix in view orientation (block b at blk_offset(D, b), rows
// of s entries; dense at 0), complex64, as M or M^dagger.
__device__ __forceinline__ void tl_stage(float2* Ms, const double2* __restrict__ mat, const TileOp& op, int D,
                                         int adjoint) {
  if (op.layout == LAYOUT_DENSE) {
    for (int idx = threadIdx.x; idx < D * D; idx += blockDim.x) {
      const int w = idx / D, u = idx - w * D;
      double2 m = adjoint ? mat[u * D + w] : mat[w * D + u];
      if (adjoint) m.y = -m.y;
      Ms[idx] = make_float2((float)m.x, (float)m.y);
    }
    return;
  }
  const int nb = 2 * D - 1, total = blk_total(D);
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    int b = 0;
    while (b + 1 < nb && idx >= blk_offset(D, b + 1)) ++b;
    const int s = blk_size(D, b);
    const int e = idx - blk_offset(D, b);
    const int w = e / s, u = e - w * s;
    int a = w, c = u;
    if (adjoint) { a = u; c = w; }
    int moff;
    if (op.layout == LAYOUT_SUM) {
      if (op.swap) { a = s - 1 - a; c = s - 1 - c; }
      moff = blk_offset(D, b);
    } else {
      moff = blk_offset(D, op.swap ? 2 * D - 2 - b : b);
    }
    double2 m = mat[moff + a * s + c];
    if (adjoint) m.y = -m.y;
    Ms[idx] = make_float2((float)m.x, (float)m.y);
  }
}

// one fibre: x[u] at X[(base + u*step)*TC + col], u < s, replaced by M x
// (rows of s entries at M; entries past a row are multiplied by zero)
template <int SB>
__device__ __forceinline__ void tl_fiber(float2* X, int TC, int col, int base, int step, int s, const float2* M) {
  f32x2 re[SB], im[SB];
#pragma unroll
  for (int u = 0; u < SB; ++u) {
    const float2 v = u < s ? X[(base + u * step) * TC + col] : make_float2(0.f, 0.f);
    re[u] = pk2(v.x, v.x);
    im[u] = pk2(v.y, v.y);
  }
#pragma unroll 1
  for (int w = 0; w < s; ++w) {
    const f32x2* m = reinterpret_cast<const f32x2*>(M + w * s);
    f32x2 P = 0ull, Q = 0ull;
#pragma unroll
    for (int u = 0; u < SB; ++u) {
      P = ffma2(m[u], re[u], P);
      Q = ffma2(m[u], im[u], Q);
    }
    const float2 p = upk2(P), q = upk2(Q);
    X[(base + w * step) * TC + col] = make_float2(p.x - q.y, p.y + q.x);
  }
}

template <int DMAX>
__device__ __forceinline__ void tl_fiber_any(float2* X, int TC, int col, int base, int step, int s, const float2* M) {
  if (s <= 4) tl_fiber<4>(X, TC, col, base, step, s, M);
  else if (DMAX > 4 && s <= 8) tl_fiber<(DMAX > 4 ? 8 : 4)>(X, TC, col, base, step, s, M);
  else if (DMAX > 8 && s <= 12) tl_fiber<(DMAX > 8 ? 12 : 4)>(X, TC, col, base, step, s, M);
  else if (DMAX > 12) tl_fiber<(DMAX > 12 ? 16 : 4)>(X, TC, col, base, step, s, M);
}

// apply op (staged in Ms) to every fibre of the tile X
template <int DMAX>
__device__ __forceinline__ void tl_apply(float2* X, const float2* Ms, const TileOp& op, int D, int TC) {
  if (op.layout == LAYOUT_DENSE) {
    const int ta = op.ta;
    const int x = ta == 0 ? 1 : 0, y = ta == 2 ? 1 : 2;
    const int esx = tl_es(D, x), esy = tl_es(D, y), step = tl_es(D, ta);
    const int nf = D * D * TC;
    for (int f = threadIdx.x; f < nf; f += blockDim.x) {
      const int col = f % TC, r = f / TC;
      const int o1 = r / D, o2 = r - o1 * D;
      tl_fiber_any<DMAX>(X, TC, col, o1 * esx + o2 * esy, step, D, Ms);
    }
    return;
  }
  const int esa = tl_es(D, op.ta), esb = tl_es(D, op.tb), esc = tl_es(D, 3 - op.ta - op.tb);
  const int nf = (2 * D - 1) * D * TC;
  for (int f = threadIdx.x; f < nf; f += blockDim.x) {
    const int col = f % TC, r = f / TC;
    const int b = r / D, ic = r - b * D;
    int base, step, s;
    tl_block(D, op.layout, b, esa, esb, base, step, s);
    tl_fiber_any<DMAX>(X, TC, col, base + ic * esc, step, s, Ms + blk_offset(D, b));
  }
}

// global offset of tile element e (t0 slowest) and column bases of a chunk
__device__ __forceinline__ void tl_offsets(int* goff, const TileGroupArg& g) {
  const int D = g.D;
  for (int e = threadIdx.x; e < g.T; e += blockDim.x) {
    const int i2 = e % D, i1 = (e / D) % D, i0 = e / (D * D);
    goff[e] = (int)(i0 * g.S[0] + i1 * g.S[1] + i2 * g.S[2]);
  }
}

__device__ __forceinline__ void tl_bases(int64_t* cb, const TileGroupArg& g, int64_t q) {
  for (int c = threadIdx.x; c < g.TC; c += blockDim.x) {
    int64_t j = q * g.TC + c, base = 0;
    if (j >= g.ncols) { cb[c] = -1; continue; }
    for (int k = g.nrest - 1; k >= 0; --k) {
      const int64_t d = j % g.D;
      j /= g.D;
      base += d * g.rest_stride[k];
    }
    cb[c] = base;
  }
}

// copy a chunk's tiles in (load) or out (store), in the order that keeps a
// warp's global addresses consecutive
__device__ __forceinline__ void tl_load(float2* X, const float2* __restrict__ src, const TileGroupArg& g,
                                        const int* goff, const int64_t* cb) {
  const int n = g.T * g.TC;
  for (int f = threadIdx.x; f < n; f += blockDim.x) {
    int col, e;
    if (g.c_fast) { col = f % g.TC; e = f / g.TC; }
    else { e = f % g.T; col = f / g.T; }
    const int64_t b = cb[col];
    X[e * g.TC + col] = b >= 0 ? src[b + goff[e]] : make_float2(0.f, 0.f);
  }
}

__device__ __forceinline__ void tl_store(float2* __restrict__ dst, const float2* X, const TileGroupArg& g,
                                         const int* goff, const int64_t* cb) {
  const int n = g.T * g.TC;
  for (int f = threadIdx.x; f < n; f += blockDim.x) {
    int col, e;
    if (g.c_fast) { col = f % g.TC; e = f / g.TC; }
    else { e = f % g.T; col = f / g.T; }
    const int64_t b = cb[col];
    if (b >= 0) dst[b + goff[e]] = X[e * g.TC + col];
  }
}

// shared-memory layout (bytes): goff, column bases, matrix, fibre-group
// sums of the adjoint's C pass (at most 2 * TL_THREADS slots), tiles
struct TlSmem {
  int goff, cb, ms, red, x, p, total;
};
__host__ __device__ __forceinline__ int tl_al(int v) { return (v + 15) & ~15; }
__host__ __device__ __forceinline__ TlSmem tl_smem(int T, int TC, int D, int adjoint) {
  TlSmem s;
  s.goff = 0;
  s.cb = tl_al(T * 4);
  s.ms = tl_al(s.cb + TC * 8);
  // + the padding a body of 16 reads past the last row
  const int ms_entries = (D * D > blk_total(D) ? D * D : blk_total(D)) + 16;
  s.red = tl_al(s.ms + ms_entries * 8);
  s.x = adjoint ? tl_al(s.red + 2 * TL_THREADS * 8) : s.red;
  s.p = tl_al(s.x + T * TC * 8);
  s.total = adjoint ? tl_al(s.p + T * TC * 8) : s.p;
  return s;
}

template <int DMAX>
__global__ void __launch_bounds__(kTlThreads) tile_forward_kernel(const float2* __restrict__ in, float2* states,
                                                                  const __grid_constant__ TileGroupArg g,
                                                                  const double2* __restrict__ arena, BatchArg bt) {
  extern __shared__ __align__(16) unsigned char smem[];
  const TlSmem L = tl_smem(g.T, g.TC, g.D, 0);
  int* goff = reinterpret_cast<int*>(smem + L.goff);
  int64_t* cb = reinterpret_cast<int64_t*>(smem + L.cb);
  float2* Ms = reinterpret_cast<float2*>(smem + L.ms);
  float2* X = reinterpret_cast<float2*>(smem + L.x);
  in += blockIdx.z * bt.state_stride;
  states += blockIdx.z * bt.state_stride;
  arena += blockIdx.z * bt.mat_stride;
  const int ms_entries = std::max(g.D * g.D, blk_total(g.D)) + 16;
  for (int i = threadIdx.x; i < ms_entries; i += blockDim.x) Ms[i] = make_float2(0.f, 0.f);
  tl_offsets(goff, g);
  pdl_wait();
  pdl_launch_dependents();
  for (int64_t q = blockIdx.x; q < g.nchunks; q += gridDim.x) {
    __syncthreads();  // previous chunk's stores done with X and cb
    tl_bases(cb, g, q);
    __syncthreads();
    tl_load(X, in, g, goff, cb);
    for (int k = 0; k < g.nops; ++k) {
      const TileOp& op = g.ops[k];
      tl_stage(Ms, arena + op.m_off, op, g.D, 0);
      __syncthreads();  // tile loaded / previous op done; matrix staged
      tl_apply<DMAX>(X, Ms, op, g.D, g.TC);
      __syncthreads();
      if (op.store_slot >= 0) tl_store(states + op.store_slot * g.slot_elems, X, g, goff, cb);
    }
  }
}

template <int DMAX>
__global__ void __launch_bounds__(kTlThreads) tile_adjoint_kernel(
    const float2* __restrict__ state_in, const float2* __restrict__ states, const float2* __restrict__ lam_out,
    float2* __restrict__ lam_in, const __grid_constant__ TileGroupArg g, const double2* __restrict__ arena,
    double2* __restrict__ cpart, BatchArg bt) {
  extern __shared__ __align__(16) unsigned char smem[];
  const TlSmem SL = tl_smem(g.T, g.TC, g.D, 1);
  int* goff = reinterpret_cast<int*>(smem + SL.goff);
  int64_t* cb = reinterpret_cast<int64_t*>(smem + SL.cb);
  float2* Ms = reinterpret_cast<float2*>(smem + SL.ms);
  float2* red = reinterpret_cast<float2*>(smem + SL.red);
  float2* Lt = reinterpret_cast<float2*>(smem + SL.x);
  float2* Pt = reinterpret_cast<float2*>(smem + SL.p);
  const int D = g.D, TC = g.TC;
  state_in += blockIdx.z * bt.state_stride;
  states += blockIdx.z * bt.state_stride;
  lam_out += blockIdx.z * bt.state_stride;
  lam_in += blockIdx.z * bt.state_stride;
  arena += blockIdx.z * bt.mat_stride;
  cpart += blockIdx.z * bt.part_stride;
  const int ms_entries = std::max(D * D, blk_total(D)) + 16;
  for (int i = threadIdx.x; i < ms_entries; i += blockDim.x) Ms[i] = make_float2(0.f, 0.f);
  tl_offsets(goff, g);
  const int64_t q = blockIdx.x;  // one chunk per CTA
  tl_bases(cb, g, q);
  __syncthreads();
  pdl_wait();
  pdl_launch_dependents();
  tl_load(Lt, lam_out, g, goff, cb);
  for (int k = g.nops - 1; k >= 0; --k) {
    const TileOp& op = g.ops[k];
    const float2* psi = op.in_slot < 0 ? state_in : states + op.in_slot * g.slot_elems;
    tl_load(Pt, psi, g, goff, cb);
    tl_stage(Ms, arena + op.m_off, op, D, 1);
    __syncthreads();
    // C partial: slot i = entry e (stored order) summed over fibre group grp
    const int nent = op.nent;
    const int G = op.G;
    const int nslot = nent * G;
    const bool dense = op.layout == LAYOUT_DENSE;
    double2* mypart = cpart + op.cpart_off + (int64_t)blockIdx.x * nent;
    // fibres of an entry: dense -> (o1, o2, col) over the two other axes;
    // block -> (ic, col) along the third axis
    int esx = 0, esy = 0, esc = 0, esa = 0, esb = 0;
    if (dense) {
      const int ta = op.ta;
      esx = tl_es(D, ta == 0 ? 1 : 0);
      esy = tl_es(D, ta == 2 ? 1 : 2);
    } else {
      esa = tl_es(D, op.ta);
      esb = tl_es(D, op.tb);
      esc = tl_es(D, 3 - op.ta - op.tb);
    }
    const int nfib = dense ? D * D * TC : D * TC;
    for (int i = threadIdx.x; i < nslot; i += blockDim.x) {
      const int e = i % nent, grp = i / nent;
      int pu, pw;
      if (dense) {
        const int u = e / D, w = e - u * D;
        const int step = tl_es(D, op.ta);
        pu = u * step;
        pw = w * step;
      } else {
        int bs = 0;
        while (bs + 1 < 2 * D - 1 && e >= blk_offset(D, bs + 1)) ++bs;
        const int s = blk_size(D, bs), r = e - blk_offset(D, bs);
        int a = r / s, c = r - a * s;
        int b = bs;
        if (op.layout == LAYOUT_SUM) {
          if (op.swap) { a = s - 1 - a; c = s - 1 - c; }
        } else if (op.swap) {
          b = 2 * D - 2 - bs;
        }
        int base, step, ss;
        tl_block(D, op.layout, b, esa, esb, base, step, ss);
        pu = base + a * step;
        pw = base + c * step;
      }
      float2 acc = make_float2(0.f, 0.f);
      for (int f = grp; f < nfib; f += G) {
        const int col = f % TC, r = f / TC;
        int fo;
        if (dense) {
          const int o1 = r / D, o2 = r - o1 * D;
          fo = o1 * esx + o2 * esy;
        } else {
          fo = r * esc;
        }
        const float2 l = Lt[(pu + fo) * TC + col], p = Pt[(pw + fo) * TC + col];
        cfma_conj(acc, l, p);
      }
      if (G == 1) mypart[e] = to_d(acc);
      else red[i] = acc;
    }
    __syncthreads();
    if (G > 1) {
      for (int e = threadIdx.x; e < nent; e += blockDim.x) {
        double2 sum = make_double2(0.0, 0.0);
        for (int q2 = 0; q2 < G; ++q2) {
          const float2 v = red[q2 * nent + e];
          sum.x += v.x;
          sum.y += v.y;
        }
        mypart[e] = sum;
      }
    }
    // lam_in = M^dagger lam_out for this op, in place
    tl_apply<DMAX>(Lt, Ms, op, D, TC);
    __syncthreads();
  }
  tl_store(lam_in, Lt, g, goff, cb);
}

template <int DMAX>
int tl_forward_t(const TileGroupArg& g, const void* in, void* states, const double2* arena, int grid, cudaStream_t st,
                 const BatchArg& bt) {
  const size_t sm = (size_t)tl_smem(g.T, g.TC, g.D, 0).total;
  auto k = tile_forward_kernel<DMAX>;
  if (sm > 48 * 1024) FOCK_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  FOCK_CUDA_TRY(launch_kernel(k, dim3(grid, 1, bt.nb), dim3(kTlThreads), sm, st, bt.pdl, (const float2*)in,
                              (float2*)states, g, arena, bt));
  return FOCK_OK;
}

template <int DMAX>
int tl_adjoint_t(const TileGroupArg& g, const void* state_in, const void* states, const void* lam_out, void* lam_in,
                 const double2* arena, double2* cpart, cudaStream_t st, const BatchArg& bt) {
  // the C slots of a dense op's fibre groups use the shared region after the matrix
  const TlSmem L = tl_smem(g.T, g.TC, g.D, 1);
  size_t sm = (size_t)L.total;
  auto k = tile_adjoint_kernel<DMAX>;
  if (sm > 48 * 1024) FOCK_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  FOCK_CUDA_TRY(launch_kernel(k, dim3((unsigned)g.nchunks, 1, bt.nb), dim3(kTlThreads), sm, st, bt.pdl,
                              (const float2*)state_in, (const float2*)states, (const float2*)lam_out, (float2*)lam_in,
                              g, arena, cpart, bt));
  return FOCK_OK;
}

}  // namespace

size_t tile_smem_bytes(int D, int TC, int adjoint) { return (size_t)tl_smem(D * D * D, TC, D, adjoint).total; }

int tile_group_g(int layout, int D, int TC) {
  // fibre groups of the adjoint's C pass: enough slots to occupy the CTA when
  // the op has few C entries (a dense op); slots <= 2 * TL_THREADS
  const int nent = layout == LAYOUT_DENSE ? D * D : blk_total(D);
  const int nfib = layout == LAYOUT_DENSE ? D * D * TC : D * TC;
  int G = std::max(1, std::min(8, (2 * kTlThreads) / nent));
  return std::min(G, nfib);
}

int launch_tile_forward(const TileGroupArg& g, const void* in, void* states, const double2* arena, int grid,
                        cudaStream_t st, const BatchArg& bt) {
  switch (dmax_bucket(g.D)) {
    case 4: return tl_forward_t<4>(g, in, states, arena, grid, st, bt);
    case 8: return tl_forward_t<8>(g, in, states, arena, grid, st, bt);
    case 12: return tl_forward_t<12>(g, in, states, arena, grid, st, bt);
    case 16: return tl_forward_t<16>(g, in, states, arena, grid, st, bt);
    default: return fock_set_error(FOCK_ERR_UNSUPPORTED, "no tile kernel for cutoff %d", g.D);
  }
}

int launch_tile_adjoint(const TileGroupArg& g, const void* state_in, const void* states, const void* lam_out,
                        void* lam_in, const double2* arena, double2* cpart, cudaStream_t st, const BatchArg& bt) {
  switch (dmax_bucket(g.D)) {
    case 4: return tl_adjoint_t<4>(g, state_in, states, lam_out, lam_in, arena, cpart, st, bt);
    case 8: return tl_adjoint_t<8>(g, state_in, states, lam_out, lam_in, arena, cpart, st, bt);
    case 12: return tl_adjoint_t<12>(g, state_in, states, lam_out, lam_in, arena, cpart, st, bt);
    case 16: return tl_adjoint_t<16>(g, state_in, states, lam_out, lam_in, arena, cpart, st, bt);
    default: return fock_set_error(FOCK_ERR_UNSUPPORTED, "no tile kernel for cutoff %d", g.D);
  }
}
