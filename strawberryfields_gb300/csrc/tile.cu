// Fused op groups of the forward sweep on a three-mode tile held in shared
// memory (pure states, complex64).
//
// A state small enough to stay in L2 (the 6-mode cutoff-12 ket is 24 MB)
// spends much of a one-op launch in ramp-up, tail and latency.  Consecutive
// ops whose modes all lie in one set of three modes {t0 < t1 < t2} form a
// group: the state is then a set of independent columns (the indices of the
// other modes), each holding a D^3 tile, and one launch applies every op of
// the group to the tiles it holds in shared memory -- the state is read once
// per group instead of once per op.  Each op's output is still written where
// the sweep keeps it (every op's output when the adjoint sweep needs them, or
// only the checkpoints and the group's last output), so the adjoint sweep's
// per-op kernels read the same stored states.
//
// A CTA takes TC consecutive columns (TC a power of two), copies their tiles
// into shared memory (lanes over columns when the innermost mode is not in the
// tile, else over the tile's contiguous innermost axis), and for each op
// stages the op's matrix (FP64 -> complex64) and applies it to every fibre:
// a dense D x D matrix along one tile axis, or the photon-number blocks of a
// two-mode op along a pair of tile axes (the selection rules of
// strawberryfields/backends/fockbackend/circuit.py:219-365).  Index
// decompositions come from tables built once per CTA (quotients by D, the
// block of every staged matrix entry, block offsets) and per op (each block's
// first element, step and size), so the fibre loop does no integer division.
#include "apply.cuh"

#include <string.h>

#include <algorithm>

namespace {

constexpr int kTlThreads = TL_THREADS;
constexpr int kMaxBlk = 2 * 16 - 1;  // blocks of a cutoff-16 two-mode op

// tile-element stride of tile axis a (0: slowest)
__host__ __device__ __forceinline__ int tl_es(int D, int a) { return a == 0 ? D * D : (a == 1 ? D : 1); }

struct BlkGeo {
  short base, step, s, pad;
};

// shared-memory layout (bytes)
struct TlSmem {
  int goff, rdiv, ent, boff, geo, ms, cb, x, total;
};
__host__ __device__ __forceinline__ int tl_al(int v) { return (v + 15) & ~15; }
__host__ __device__ __forceinline__ TlSmem tl_smem(int D, int TC) {
  TlSmem s;
  const int T = D * D * D, nb = 2 * D - 1, total = blk_total(D);
  const int ms_entries = (D * D > total ? D * D : total) + 16;  // + what a body of 16 reads past a row
  s.goff = 0;
  s.rdiv = tl_al(T * 4);
  s.ent = tl_al(s.rdiv + nb * D * 2);
  s.boff = tl_al(s.ent + total * 2);
  s.geo = tl_al(s.boff + (nb + 1) * 4);
  s.ms = tl_al(s.geo + kMaxBlk * (int)sizeof(BlkGeo));
  s.cb = tl_al(s.ms + ms_entries * 8);
  s.x = tl_al(s.cb + TC * 8);
  s.total = tl_al(s.x + T * TC * 8);
  return s;
}

// one fibre: x[u] at X[((base + u*step) << lg) | col], u < s, replaced by
// M x (rows of s entries at M; entries past a row are multiplied by zero)
template <int SB>
__device__ __forceinline__ void tl_fiber(float2* X, int lg, int col, int base, int step, int s, const float2* M) {
  f32x2 re[SB], im[SB];
#pragma unroll
  for (int u = 0; u < SB; ++u) {
    const float2 v = u < s ? X[((base + u * step) << lg) | col] : make_float2(0.f, 0.f);
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
    X[((base + w * step) << lg) | col] = make_float2(p.x - q.y, p.y + q.x);
  }
}

template <int DMAX>
__device__ __forceinline__ void tl_fiber_any(float2* X, int lg, int col, int base, int step, int s, const float2* M) {
  if (s <= 4) tl_fiber<4>(X, lg, col, base, step, s, M);
  else if (DMAX > 4 && s <= 8) tl_fiber<(DMAX > 4 ? 8 : 4)>(X, lg, col, base, step, s, M);
  else if (DMAX > 8 && s <= 12) tl_fiber<(DMAX > 8 ? 12 : 4)>(X, lg, col, base, step, s, M);
  else if (DMAX > 12) tl_fiber<(DMAX > 12 ? 16 : 4)>(X, lg, col, base, step, s, M);
}

template <int DMAX>
__global__ void __launch_bounds__(kTlThreads) tile_forward_kernel(const float2* __restrict__ in, float2* states,
                                                                  const __grid_constant__ TileGroupArg g,
                                                                  const double2* __restrict__ arena, BatchArg bt) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int D = g.D, T = g.T, TC = g.TC, lg = g.lgTC, nb = 2 * D - 1, total = blk_total(D);
  const TlSmem L = tl_smem(D, TC);
  int* goff = reinterpret_cast<int*>(smem + L.goff);
  unsigned short* rdiv = reinterpret_cast<unsigned short*>(smem + L.rdiv);
  unsigned short* ent = reinterpret_cast<unsigned short*>(smem + L.ent);
  int* boff = reinterpret_cast<int*>(smem + L.boff);
  BlkGeo* geo = reinterpret_cast<BlkGeo*>(smem + L.geo);
  float2* Ms = reinterpret_cast<float2*>(smem + L.ms);
  int64_t* cb = reinterpret_cast<int64_t*>(smem + L.cb);
  float2* X = reinterpret_cast<float2*>(smem + L.x);
  in += blockIdx.z * bt.state_stride;
  states += blockIdx.z * bt.state_stride;
  arena += blockIdx.z * bt.mat_stride;

  // tables (depend on D and the tile modes only)
  for (int e = threadIdx.x; e < T; e += blockDim.x) {
    const int i2 = e % D, i1 = (e / D) % D, i0 = e / (D * D);
    goff[e] = (int)(i0 * g.S[0] + i1 * g.S[1] + i2 * g.S[2]);
  }
  for (int r = threadIdx.x; r < nb * D; r += blockDim.x) rdiv[r] = (unsigned short)(((r / D) << 8) | (r % D));
  for (int b = threadIdx.x; b <= nb; b += blockDim.x) boff[b] = b < nb ? blk_offset(D, b) : total;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    const int s = blk_size(D, b), o = blk_offset(D, b);
    for (int e = 0; e < s * s; ++e) ent[o + e] = (unsigned short)((b << 8) | ((e / s) << 4) | (e % s));
  }
  const int ms_entries = (D * D > total ? D * D : total) + 16;
  for (int i = threadIdx.x; i < ms_entries; i += blockDim.x) Ms[i] = make_float2(0.f, 0.f);
  pdl_wait();
  pdl_launch_dependents();

  for (int64_t q = blockIdx.x; q < g.nchunks; q += gridDim.x) {
    __syncthreads();  // tables ready; the previous chunk's stores are done with X and cb
    for (int c = threadIdx.x; c < TC; c += blockDim.x) {
      int64_t j = q * TC + c, base = 0;
      if (j >= g.ncols) {
        cb[c] = -1;
        continue;
      }
      for (int k = g.nrest - 1; k >= 0; --k) {
        const int64_t d = j % D;
        j /= D;
        base += d * g.rest_stride[k];
      }
      cb[c] = base;
    }
    __syncthreads();
    // load: lanes over columns (c_fast) or over the contiguous innermost tile axis
    for (int f = threadIdx.x; f < T * TC; f += blockDim.x) {
      int col, e;
      if (g.c_fast) { col = f & (TC - 1); e = f >> lg; }
      else { e = f % T; col = f / T; }
      const int64_t b = cb[col];
      X[(e << lg) | col] = b >= 0 ? in[b + goff[e]] : make_float2(0.f, 0.f);
    }
    for (int k = 0; k < g.nops; ++k) {
      const TileOp& op = g.ops[k];
      const double2* mat = arena + op.m_off;
      const bool dense = op.layout == LAYOUT_DENSE;
      int esa = 0, esb = 0, esc = 0, esx = 0, esy = 0;
      if (dense) {
        esx = tl_es(D, op.ta == 0 ? 1 : 0);
        esy = tl_es(D, op.ta == 2 ? 1 : 2);
        esa = tl_es(D, op.ta);
        for (int idx = threadIdx.x; idx < D * D; idx += blockDim.x) {
          const double2 m = mat[idx];  // row-major [out][in]: the view order already
          Ms[idx] = make_float2((float)m.x, (float)m.y);
        }
      } else {
        esa = tl_es(D, op.ta);
        esb = tl_es(D, op.tb);
        esc = tl_es(D, 3 - op.ta - op.tb);
        const int sum = op.layout == LAYOUT_SUM;
        for (int b = threadIdx.x; b < nb; b += blockDim.x) {
          BlkGeo gb;
          const int delta = b - (D - 1);
          const int lo = delta > 0 ? delta : 0;
          gb.s = (short)blk_size(D, b);
          if (sum) {
            gb.base = (short)(lo * esa + (b - lo) * esb);
            gb.step = (short)(esa - esb);
          } else {
            gb.base = (short)(lo * esa + (lo - delta) * esb);
            gb.step = (short)(esa + esb);
          }
          gb.pad = 0;
          geo[b] = gb;
        }
        for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
          const int t = ent[idx];
          const int b = t >> 8, w = (t >> 4) & 15, u = t & 15;
          const int s = blk_size(D, b);
          int a = w, c = u, moff;
          if (sum) {
            if (op.swap) { a = s - 1 - a; c = s - 1 - c; }
            moff = boff[b];
          } else {
            moff = boff[op.swap ? 2 * D - 2 - b : b];
          }
          const double2 m = mat[moff + a * s + c];
          Ms[idx] = make_float2((float)m.x, (float)m.y);
        }
      }
      __syncthreads();  // tile loaded / previous op done; matrix and geometry staged
      if (dense) {
        const int nf = (D * D) << lg;
        for (int f = threadIdx.x; f < nf; f += blockDim.x) {
          const int col = f & (TC - 1), qd = rdiv[f >> lg];
          tl_fiber_any<DMAX>(X, lg, col, (qd >> 8) * esx + (qd & 255) * esy, esa, D, Ms);
        }
      } else {
        const int nf = (nb * D) << lg;
        for (int f = threadIdx.x; f < nf; f += blockDim.x) {
          const int col = f & (TC - 1), qd = rdiv[f >> lg];
          const int b = qd >> 8, ic = qd & 255;
          const BlkGeo gb = geo[b];
          tl_fiber_any<DMAX>(X, lg, col, gb.base + ic * esc, gb.step, gb.s, Ms + boff[b]);
        }
      }
      __syncthreads();
      if (op.store_slot >= 0) {
        float2* dst = states + op.store_slot * g.slot_elems;
        for (int f = threadIdx.x; f < T * TC; f += blockDim.x) {
          int col, e;
          if (g.c_fast) { col = f & (TC - 1); e = f >> lg; }
          else { e = f % T; col = f / T; }
          const int64_t b = cb[col];
          if (b >= 0) dst[b + goff[e]] = X[(e << lg) | col];
        }
      }
    }
  }
}

template <int DMAX>
int tl_forward_t(const TileGroupArg& g, const void* in, void* states, const double2* arena, int grid, cudaStream_t st,
                 const BatchArg& bt) {
  const size_t sm = (size_t)tl_smem(g.D, g.TC).total;
  auto k = tile_forward_kernel<DMAX>;
  if (sm > 48 * 1024) FOCK_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  FOCK_CUDA_TRY(launch_kernel(k, dim3(grid, 1, bt.nb), dim3(kTlThreads), sm, st, bt.pdl, (const float2*)in,
                              (float2*)states, g, arena, bt));
  return FOCK_OK;
}

}  // namespace

size_t tile_smem_bytes(int D, int TC) { return (size_t)tl_smem(D, TC).total; }

int launch_tile_forward(const TileGroupArg& g, const void* in, void* states, const double2* arena, int grid,
                        cudaStream_t st, const BatchArg& bt) {
  if (g.D > 16 || g.TC < 1 || (g.TC & (g.TC - 1)) || g.nops < 1 || g.nops > TL_MAX_OPS)
    return fock_set_error(FOCK_ERR_INVALID, "bad tile group (cutoff %d, %d columns, %d ops)", g.D, g.TC, g.nops);
  switch (dmax_bucket(g.D)) {
    case 4: return tl_forward_t<4>(g, in, states, arena, grid, st, bt);
    case 8: return tl_forward_t<8>(g, in, states, arena, grid, st, bt);
    case 12: return tl_forward_t<12>(g, in, states, arena, grid, st, bt);
    case 16: return tl_forward_t<16>(g, in, states, arena, grid, st, bt);
    default: return fock_set_error(FOCK_ERR_UNSUPPORTED, "no tile kernel for cutoff %d", g.D);
  }
}
