// Plane-tile kernels: gate apply and adjoint step over whole column planes.
//
// A one-mode op sees the state as [A][D][C] and a two-mode op as
// [A][D][B][D][C]; the D (one mode) or D x D (two modes) elements that share
// a column j = (a, b, c) form that column's plane.  A persistent CTA takes
// tiles of TC consecutive columns and
//   1. copies the tile's planes into shared memory with cp.async, in the
//      order that keeps global addresses consecutive across a warp (lanes
//      over columns when the innermost axis C is long, lanes over plane
//      elements when C is short -- e.g. a beamsplitter on the last two modes,
//      whose planes are contiguous 2-D blocks);
//   2. applies every photon-number block of the op to every column from
//      shared memory (warp = one block for 32 columns; each lane holds one
//      column's block in registers, the block matrix is broadcast from
//      shared memory);
//   3. writes the tile back in the same coalesced order.
// Every state element therefore crosses HBM exactly once per op whatever
// the mode pair, the block matrices are staged once per CTA rather than once
// per (block, column tile), and the next tile's copies are in flight while
// the current one is computed (two buffers in the apply kernel).
//
// The adjoint kernel holds lam_out and psi_in tiles.  Its C accumulation
// deals the C entries (block y, row u, column w) out to the threads in equal
// shares -- thread t owns entries t, t + 256, ... and sums
// conj(lam[u]) psi[w] over the tile's columns in registers (or over one of G
// column groups when there are fewer entries than threads), so no thread waits
// at the barrier for the large blocks' rows; consecutive threads hold
// consecutive w of one row, so the lam value is a broadcast and the psi values
// of a half-warp fall in distinct banks.  Then lam_in = M^dagger lam_out is
// formed in place with the apply mapping and written back.  Per-CTA partial
// sums of C go to cpart[CTA][entries] (FP64, stored orientation) for a
// fixed-order reduction.
//
// The block structure is the reference's selection rules
// (strawberryfields/backends/fockbackend/circuit.py:219-365): sum blocks for
// beamsplitter / MZ, difference blocks for two-mode squeezing and the loss
// superoperator, one dense block for single-mode gates.
#include "apply.cuh"

#include <algorithm>
#include <map>
#include <mutex>
#include <string.h>
#include <tuple>
#include <vector>

__device__ __forceinline__ void pl_cp(float2* dst, const float2* src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(src));
}
__device__ __forceinline__ void pl_cp(double2* dst, const double2* src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(src));
}
__device__ __forceinline__ void pl_commit() { asm volatile("cp.async.commit_group;\n" ::); }

// Blocks of size s run the unrolled body of size pl_pad(s) (s rounded up to a
// multiple of PL_S_STEP), and are staged at that size with zero padding: half
// the bodies of one body per size.  The warps of a tile apply blocks of
// different sizes at once, and with one body per size the kernels stalled on
// instruction fetch more than on anything else (GB300, cutoff 12: 1.8 and 3.3
// fetch stalls per issued instruction in the adjoint and apply).  Steps of 2
// measured faster than steps of 4 (fewer padded FMAs) on the QNN step.
#ifndef PL_S_STEP
#define PL_S_STEP 2
#endif
__host__ __device__ __forceinline__ int pl_pad(int s) { return (s + PL_S_STEP - 1) / PL_S_STEP * PL_S_STEP; }
template <int N>
__device__ __forceinline__ void pl_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// C sub-blocks (PL_RT x PL_RT) of the largest plane with blocks up to smax,
// and the sub-blocks per thread of the C pass that covers them
__host__ __device__ constexpr int pl_ceil_rt(int s) { return (s + PL_RT - 1) / PL_RT; }
__host__ __device__ constexpr int pl_citems_max(int smax) {
  int n = 0;
  if (smax <= PL_MAX_D2) {
    for (int s = 1; s <= smax; ++s) n += 2 * pl_ceil_rt(s) * pl_ceil_rt(s);
    n -= pl_ceil_rt(smax) * pl_ceil_rt(smax);
  } else {
    n = pl_ceil_rt(smax) * pl_ceil_rt(smax);
  }
  return n;
}
__host__ __device__ constexpr int pl_ki(int smax) { return (pl_citems_max(smax) + PL_THREADS - 1) / PL_THREADS; }

// columns of a tile that starts at column j0 (the last tile may be partial)
__device__ __forceinline__ int pl_cols(int64_t tc, int64_t rest) { return (int)(rest < tc ? rest : tc); }

__device__ __forceinline__ int64_t pl_col_base(const PlaneGeom& g, int64_t j) {
  const int64_t c = j % g.C;
  const int64_t t = j / g.C;
  const int64_t b = t % g.B;
  const int64_t a = t / g.B;
  return a * (g.s1 * g.D) + b * (g.s2 * g.D) + c;
}

// global offsets of the plane elements (e = i*D + k, or e = i for one mode)
__device__ __forceinline__ void pl_offsets(int64_t* goff, const PlaneGeom& g) {
  for (int e = threadIdx.x; e < g.E; e += PL_THREADS)
    goff[e] = g.two ? (int64_t)(e / g.D) * g.s1 + (int64_t)(e % g.D) * g.s2 : (int64_t)e * g.s1;
}

// column bases of tile t (the 64-bit index decomposition runs once per
// column here, not once per copied element)
__device__ __forceinline__ void pl_bases(int64_t* cb, const PlaneGeom& g, int64_t t) {
  if (t >= g.ntiles) return;
  const int64_t j0 = t * g.TC;
  for (int cc = threadIdx.x; cc < g.TC; cc += PL_THREADS)
    if (j0 + cc < g.ncols) cb[cc] = pl_col_base(g, j0 + cc);
}

// column of flat tile index idx (idx / E by multiply-shift; exact for
// idx < 2^16 and E <= 1024)
__device__ __forceinline__ int pl_fcol(const PlaneGeom& g, int idx) {
  return (int)(((uint64_t)(unsigned)idx * (uint64_t)g.emagic) >> 26);
}

// Issue the copies of the tile's tcv columns (bases cb) into T (row stride EP).
// Flat tiles (gate on the innermost axes) are one contiguous range.
template <typename CT>
__device__ __forceinline__ void pl_issue(const CT* __restrict__ src, CT* T, const PlaneGeom& g,
                                         const int64_t* goff, const int64_t* cb, int tcv) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (g.flat) {
    const CT* s = src + cb[0];
    const int n = tcv * g.E;
    for (int idx = threadIdx.x; idx < n; idx += PL_THREADS) {
      const int col = pl_fcol(g, idx);
      pl_cp(T + col * g.EP + (idx - col * g.E), s + idx);
    }
  } else if (g.c_inner) {
    for (int cc = lane; cc < tcv; cc += 32) {
      const CT* s = src + cb[cc];
      CT* row = T + cc * g.EP;
      for (int e = warp; e < g.E; e += PL_WARPS) pl_cp(row + e, s + goff[e]);
    }
  } else {
    for (int cc = warp; cc < tcv; cc += PL_WARPS) {
      const CT* s = src + cb[cc];
      CT* row = T + cc * g.EP;
      for (int e = lane; e < g.E; e += 32) pl_cp(row + e, s + goff[e]);
    }
  }
  pl_commit();
}

template <typename CT>
__device__ __forceinline__ void pl_store(CT* __restrict__ dst, const CT* T, const PlaneGeom& g, const int64_t* goff,
                                         const int64_t* cb, int tcv) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (g.flat) {
    CT* d = dst + cb[0];
    const int n = tcv * g.E;
    for (int idx = threadIdx.x; idx < n; idx += PL_THREADS) {
      const int col = pl_fcol(g, idx);
      d[idx] = T[col * g.EP + (idx - col * g.E)];
    }
  } else if (g.c_inner) {
    for (int cc = lane; cc < tcv; cc += 32) {
      CT* d = dst + cb[cc];
      const CT* row = T + cc * g.EP;
      for (int e = warp; e < g.E; e += PL_WARPS) d[goff[e]] = row[e];
    }
  } else {
    for (int cc = warp; cc < tcv; cc += PL_WARPS) {
      CT* d = dst + cb[cc];
      const CT* row = T + cc * g.EP;
      for (int e = lane; e < g.E; e += 32) d[goff[e]] = row[e];
    }
  }
}

// Stage every block's matrix (view orientation, state precision): forward
// Ms[w][u] maps view input u to output w; with MF_ADJOINT the conjugate
// transpose.  Reverse-stored sum blocks (MF_SWAP) read s-1-position.
template <typename CT>
__device__ __forceinline__ void pl_stage(CT* Ms, const double2* __restrict__ mat, const PlaneGeom& g, int mflags) {
  const int cj = ((mflags & MF_ADJOINT) ? 1 : 0) ^ ((mflags & MF_CONJ) ? 1 : 0);
#pragma unroll 4
  for (int idx = threadIdx.x; idx < g.ms_total; idx += PL_THREADS) {
    int y = 0;
    while (y + 1 < g.nblk && idx >= g.ms_off[y + 1]) ++y;
    const int s = g.s[y], sp = pl_pad(s);
    const int e = idx - g.ms_off[y];
    const int w = e / sp, u = e - w * sp;
    if (w >= s || u >= s) {
      Ms[idx] = czero<CT>();
      continue;
    }
    int a = w, c = u;
    if (mflags & MF_ADJOINT) { a = u; c = w; }
    if (g.rev[y]) { a = s - 1 - a; c = s - 1 - c; }
    Ms[idx] = mat_entry<CT>(mat, g.moff[y] + a * s + c, cj, mflags);
  }
}

// one column's block: x = Ms x in place (positions base + u*step); complex64
// with paired FMAs (the column as (Re, Re) / (Im, Im) pairs, entries read as
// pairs)
template <typename CT, int S>
__device__ __forceinline__ void pl_block(CT* row, int base, int step, const CT* Ms, int s) {
  CT x[S];
#pragma unroll
  for (int u = 0; u < S; ++u) x[u] = u < s ? row[base + u * step] : czero<CT>();
  if constexpr (sizeof(CT) == 8) {
    f32x2 re[S], im[S];
#pragma unroll
    for (int u = 0; u < S; ++u) {
      re[u] = pk2(x[u].x, x[u].x);
      im[u] = pk2(x[u].y, x[u].y);
    }
#pragma unroll
    for (int w = 0; w < S; ++w) {
      if (w >= s) break;
      const f32x2* m = reinterpret_cast<const f32x2*>(Ms + w * S);
      f32x2 P = 0ull, Q = 0ull;
#pragma unroll
      for (int u = 0; u < S; ++u) {
        P = ffma2(m[u], re[u], P);
        Q = ffma2(m[u], im[u], Q);
      }
      const float2 p = upk2(P), q = upk2(Q);
      row[base + w * step] = CT{p.x - q.y, p.y + q.x};
    }
  } else {
#pragma unroll
    for (int w = 0; w < S; ++w) {
      if (w >= s) break;
      CT a = czero<CT>();
#pragma unroll
      for (int u = 0; u < S; ++u) cfma(a, Ms[w * S + u], x[u]);
      row[base + w * step] = a;
    }
  }
}
template <typename CT, int S, int SMAX>
struct PlBlock {
  __device__ __forceinline__ static void run(int s, CT* row, int base, int step, const CT* Ms) {
    if (s <= S) pl_block<CT, S>(row, base, step, Ms, s);
    else PlBlock<CT, S + PL_S_STEP, SMAX>::run(s, row, base, step, Ms);
  }
};
template <typename CT, int SMAX>
struct PlBlock<CT, SMAX + PL_S_STEP, SMAX> {
  __device__ __forceinline__ static void run(int, CT*, int, int, const CT*) {}
};

// step 2: every block of every column of the tile (warp items from the host)
template <typename CT, int SMAX>
__device__ __forceinline__ void pl_apply_tile(CT* T, const CT* Ms, const PlaneGeom& g, int tcv) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int it = g.warp_start[warp]; it < g.warp_start[warp + 1]; ++it) {
    const int item = g.items[it];
    const int y = item >> 4, col = (item & 15) * 32 + lane;
    if (col < tcv) PlBlock<CT, PL_S_STEP, SMAX>::run(g.s[y], T + col * g.EP, g.base[y], g.step[y], Ms + g.ms_off[y]);
  }
}

template <typename CT, int SMAX>
__global__ void __launch_bounds__(PL_THREADS, (sizeof(CT) == 8 && SMAX <= 12) ? 3 : 2)
    plane_apply_kernel(const CT* __restrict__ in, CT* __restrict__ out, const __grid_constant__ PlaneGeom g,
                       const double2* __restrict__ mat, int mflags, BatchArg bt) {
  extern __shared__ __align__(16) unsigned char smem[];
  CT* Ms = reinterpret_cast<CT*>(smem);
  int64_t* goff = reinterpret_cast<int64_t*>(smem + g.sm_goff);
  int64_t* cb0 = reinterpret_cast<int64_t*>(smem + g.sm_cb);
  CT* T0 = reinterpret_cast<CT*>(smem + g.sm_tile);
  const int64_t tsz = (int64_t)g.TC * g.EP;
  in += blockIdx.z * bt.state_stride;
  out += blockIdx.z * bt.state_stride;
  mat = mat_batch(mat, blockIdx.z * bt.mat_stride, mflags);
  const int64_t G = gridDim.x;
  int64_t t = blockIdx.x;
  pl_offsets(goff, g);
  pl_bases(cb0, g, t);
  pl_bases(cb0 + g.TC, g, t + G);
  // the matrices were built before the sweep: staged while the previous op
  // finishes
  pl_stage(Ms, mat, g, mflags);
  __syncthreads();
  pdl_wait();
  pdl_launch_dependents();
  if (t < g.ntiles) pl_issue(in, T0, g, goff, cb0, pl_cols(g.TC, g.ncols - t * g.TC));
  int buf = 0;
  // buffer buf holds tile t (bases cb0 + buf*TC); buf^1 receives tile t + G
  for (; t < g.ntiles; t += G) {
    const int64_t tn = t + G;
    const int tcv = pl_cols(g.TC, g.ncols - t * g.TC);
    CT* T = T0 + buf * tsz;
    int64_t* cb = cb0 + buf * g.TC;
    if (tn < g.ntiles) {
      pl_issue(in, T0 + (buf ^ 1) * tsz, g, goff, cb0 + (buf ^ 1) * g.TC, pl_cols(g.TC, g.ncols - tn * g.TC));
      pl_wait<1>();
    } else {
      pl_wait<0>();
    }
    __syncthreads();  // tile t (and the staged matrices) visible to all
    pl_apply_tile<CT, SMAX>(T, Ms, g, tcv);
    __syncthreads();
    pl_store(out, T, g, goff, cb, tcv);
    __syncthreads();  // buffer and bases free before they are refilled
    pl_bases(cb, g, t + 2 * G);
    __syncthreads();
    buf ^= 1;
  }
}

template <typename CT, int SMAX>
__global__ void __launch_bounds__(PL_THREADS, 2)
    plane_adjoint_kernel(const CT* __restrict__ psi_in, const CT* __restrict__ lam_out, CT* __restrict__ lam_in,
                         const __grid_constant__ PlaneGeom g, const double2* __restrict__ mat, int mflags,
                         double2* __restrict__ cpart, BatchArg bt) {
  extern __shared__ __align__(16) unsigned char smem[];
  CT* MsH = reinterpret_cast<CT*>(smem);
  int64_t* goff = reinterpret_cast<int64_t*>(smem + g.sm_goff);
  int64_t* cb0 = reinterpret_cast<int64_t*>(smem + g.sm_cb);
  CT* L = reinterpret_cast<CT*>(smem + g.sm_tile);
  CT* P = L + (int64_t)g.TC * g.EP;
  const int tid = threadIdx.x;
  psi_in += blockIdx.z * bt.state_stride;
  lam_out += blockIdx.z * bt.state_stride;
  if (lam_in) lam_in += blockIdx.z * bt.state_stride;
  mat = mat_batch(mat, blockIdx.z * bt.mat_stride, mflags);
  cpart += blockIdx.z * bt.part_stride + (int64_t)blockIdx.x * g.nent;
  const int64_t GX = gridDim.x;
  int64_t t = blockIdx.x;
  pl_offsets(goff, g);
  pl_bases(cb0, g, t);
  pl_bases(cb0 + g.TC, g, t + GX);
  // the matrices were built before the sweep: staged while the previous op
  // finishes
  if (lam_in) pl_stage(MsH, mat, g, mflags | MF_ADJOINT);
  __syncthreads();
  pdl_wait();
  pdl_launch_dependents();
  if (t < g.ntiles) {
    const int tcv = pl_cols(g.TC, g.ncols - t * g.TC);
    pl_issue(lam_out, L, g, goff, cb0, tcv);
    pl_issue(psi_in, P, g, goff, cb0, tcv);
  }

  // C pass: thread slot i = tid + k * PL_THREADS sums the PL_RT x PL_RT
  // sub-block citems[i % ncitems] of one block's C over the columns
  // col = i / ncitems (mod G) -- each shared load feeds PL_RT complex FMAs
  constexpr int KI = pl_ki(SMAX);
  const int G = g.G;
  int lb[KI], pb[KI], st[KI], nr[KI], nc[KI], grp[KI];
  CT acc[KI][PL_RT][PL_RT];
#pragma unroll
  for (int k = 0; k < KI; ++k) {
    const int i = tid + k * PL_THREADS;
    grp[k] = -1;
    lb[k] = pb[k] = st[k] = nr[k] = nc[k] = 0;
#pragma unroll
    for (int r = 0; r < PL_RT; ++r)
#pragma unroll
      for (int c = 0; c < PL_RT; ++c) acc[k][r][c] = czero<CT>();
    if (i < g.nslot) {
      const int it = g.citems[i % g.ncitems];
      const int y = it >> 10, r0 = (it >> 5) & 31, c0 = it & 31, s = g.s[y];
      st[k] = g.step[y];
      lb[k] = g.base[y] + r0 * st[k];
      pb[k] = g.base[y] + c0 * st[k];
      nr[k] = s - r0 < PL_RT ? s - r0 : PL_RT;
      nc[k] = s - c0 < PL_RT ? s - c0 : PL_RT;
      grp[k] = i / g.ncitems;
    }
  }

  // bases of tile t at cb0 + cur*TC, of tile t + GX at the other half
  int cur = 0;
  for (; t < g.ntiles; t += GX) {
    const int64_t tn = t + GX;
    const int tcv = pl_cols(g.TC, g.ncols - t * g.TC);
    int64_t* cb = cb0 + cur * g.TC;
    int64_t* cbn = cb0 + (cur ^ 1) * g.TC;
    pl_wait<0>();
    __syncthreads();
#pragma unroll
    for (int k = 0; k < KI; ++k) {
      if (grp[k] < 0) break;
      for (int col = grp[k]; col < tcv; col += G) {
        const CT* lr = L + col * g.EP + lb[k];
        const CT* pr = P + col * g.EP + pb[k];
        CT lv[PL_RT], pv[PL_RT];
#pragma unroll
        for (int r = 0; r < PL_RT; ++r) {
          lv[r] = r < nr[k] ? lr[r * st[k]] : czero<CT>();
          pv[r] = r < nc[k] ? pr[r * st[k]] : czero<CT>();
        }
#pragma unroll
        for (int r = 0; r < PL_RT; ++r)
#pragma unroll
          for (int c = 0; c < PL_RT; ++c) cfma_conj(acc[k][r][c], lv[r], pv[c]);
      }
    }
    __syncthreads();
    const int tcn = tn < g.ntiles ? pl_cols(g.TC, g.ncols - tn * g.TC) : 0;
    if (tn < g.ntiles) pl_issue(psi_in, P, g, goff, cbn, tcn);  // the psi tile is free
    if (lam_in) {
      pl_apply_tile<CT, SMAX>(L, MsH, g, tcv);
      __syncthreads();
      pl_store(lam_in, L, g, goff, cb, tcv);
      __syncthreads();
    }
    if (tn < g.ntiles) pl_issue(lam_out, L, g, goff, cbn, tcn);
    pl_bases(cb, g, tn + GX);  // tile t's bases are no longer read
    cur ^= 1;
  }
  pl_wait<0>();
  __syncthreads();
  // partial C of this CTA (stored orientation)
  auto put = [&](int it, int r, int c, double2 v) {
    const int y = it >> 10, u = ((it >> 5) & 31) + r, w = (it & 31) + c, s = g.s[y];
    if (u >= s || w >= s) return;
    const int a = g.rev[y] ? s - 1 - u : u, b = g.rev[y] ? s - 1 - w : w;
    cpart[g.cout_off[y] + a * s + b] = v;
  };
  if (G == 1) {
#pragma unroll
    for (int k = 0; k < KI; ++k) {
      if (grp[k] < 0) break;
      const int it = g.citems[(tid + k * PL_THREADS) % g.ncitems];
#pragma unroll
      for (int r = 0; r < PL_RT; ++r)
#pragma unroll
        for (int c = 0; c < PL_RT; ++c) put(it, r, c, to_d(acc[k][r][c]));
    }
  } else {
    // G > 1 only when KI = 1: sum the G column groups of each sub-block entry
    // through shared memory (fixed order)
    CT* red = L;
    if (grp[0] >= 0) {
#pragma unroll
      for (int r = 0; r < PL_RT; ++r)
#pragma unroll
        for (int c = 0; c < PL_RT; ++c) red[tid * PL_RT * PL_RT + r * PL_RT + c] = acc[0][r][c];
    }
    __syncthreads();
    for (int e = tid; e < g.ncitems * PL_RT * PL_RT; e += PL_THREADS) {
      const int item = e / (PL_RT * PL_RT), rc = e - item * PL_RT * PL_RT;
      double2 sum = make_double2(0.0, 0.0);
      for (int q = 0; q < G; ++q) {
        const double2 v = to_d(red[(q * g.ncitems + item) * PL_RT * PL_RT + rc]);
        sum.x += v.x;
        sum.y += v.y;
      }
      put(g.citems[item], rc / PL_RT, rc % PL_RT, sum);
    }
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

int make_plane_geom(int dtype, const AxisView& v, int D, int layout, int swap, int adjoint, PlaneGeom* out,
                    int tile_columns) {
  PlaneGeom g;
  memset(&g, 0, sizeof(g));
  const int esz = dtype == FOCK_C64 ? 8 : 16;
  g.two = layout != LAYOUT_DENSE;
  g.D = D;
  g.E = g.two ? D * D : D;
  if (g.two ? D > PL_MAX_D2 : D > PL_MAX_D1) return 0;
  if (g.E > PL_THREADS && g.two) return 0;
  g.EP = g.E | 1;
  g.A = v.A; g.B = v.B; g.C = v.C; g.s1 = v.s1; g.s2 = v.s2; g.ncols = v.ncols;
  g.c_inner = v.C >= 16 ? 1 : 0;
  // the gate's axes are the innermost ones: column j's plane starts at j*E
  g.flat = v.C == 1 && (!g.two || v.B == 1) ? 1 : 0;
  g.emagic = (unsigned)(((1ull << 26) + g.E - 1) / g.E);
  g.nblk = g.two ? 2 * D - 1 : 1;
  int ms = 0;
  for (int y = 0; y < g.nblk; ++y) {
    if (!g.two) {
      g.base[y] = 0; g.step[y] = 1; g.s[y] = (short)D; g.moff[y] = 0; g.rev[y] = 0; g.cout_off[y] = 0;
    } else {
      const int b = block_of_y(D, y);
      const int s = blk_size(D, b);
      g.s[y] = (short)s;
      if (layout == LAYOUT_SUM) {
        const int lo = blk_lo(D, 1, b);
        g.base[y] = (short)(lo * D + (b - lo));
        g.step[y] = (short)(D - 1);
        g.moff[y] = blk_offset(D, b);
        g.rev[y] = (unsigned char)(swap ? 1 : 0);
        g.cout_off[y] = blk_offset(D, b);
      } else {
        const int delta = b - (D - 1);
        const int lo = delta > 0 ? delta : 0;
        g.base[y] = (short)(lo * D + (lo - delta));
        g.step[y] = (short)(D + 1);
        const int bs = swap ? 2 * D - 2 - b : b;
        g.moff[y] = blk_offset(D, bs);
        g.rev[y] = 0;
        g.cout_off[y] = blk_offset(D, bs);
      }
    }
    g.ms_off[y] = ms;
    ms += pl_pad(g.s[y]) * pl_pad(g.s[y]);
    g.nent += g.s[y] * g.s[y];
  }
  g.ms_off[g.nblk] = ms;
  g.ms_total = ms;
  // C pass: PL_RT x PL_RT sub-blocks of every block's C, times G column
  // groups when there are few sub-blocks
  g.ncitems = 0;
  for (int y = 0; y < g.nblk; ++y)
    for (int r0 = 0; r0 < g.s[y]; r0 += PL_RT)
      for (int c0 = 0; c0 < g.s[y]; c0 += PL_RT) {
        if (g.ncitems >= PL_MAX_CITEMS) return 0;
        g.citems[g.ncitems++] = (unsigned short)((y << 10) | (r0 << 5) | c0);
      }
  g.G = std::max(1, PL_THREADS / g.ncitems);
  g.nslot = g.ncitems * g.G;
  if (g.nslot > PL_THREADS * pl_ki(dmax_bucket(D))) return 0;
  // columns per tile: one warp of columns per block for two modes; enough
  // column groups to give every warp a dense block otherwise
  // two-mode planes: tile_columns (8..32; default 32) -- fewer columns give
  // smaller tiles and more resident CTAs, which pays on L2-resident states
  // (the autotuner picks it per op)
  if (tile_columns && (tile_columns < 8 || tile_columns > 32)) return 0;
  g.TC = g.two ? (tile_columns ? tile_columns : 32) : 256;
  const size_t tile_cap = adjoint ? 96 * 1024 : 72 * 1024;  // both buffers
  while (g.TC > 32 && (size_t)2 * g.TC * g.EP * esz > tile_cap) g.TC >>= 1;
  g.ntiles = (g.ncols + g.TC - 1) / g.TC;
  if (g.flat && (int64_t)g.TC * g.E >= (1 << 16)) return 0;
  // warp items (block, column group), longest first onto the least loaded warp
  const int ncg = (g.TC + 31) / 32;
  std::vector<std::pair<int, int>> items;  // (cost, item)
  for (int y = 0; y < g.nblk; ++y)
    for (int c = 0; c < ncg; ++c) items.push_back({pl_pad(g.s[y]) * pl_pad(g.s[y]), (y << 4) | c});
  if ((int)items.size() > PL_MAX_ITEMS) return 0;
  std::stable_sort(items.begin(), items.end(), [](const std::pair<int, int>& a, const std::pair<int, int>& b) {
    return a.first > b.first;
  });
  std::vector<std::vector<int>> bins(PL_WARPS);
  std::vector<long> load(PL_WARPS, 0);
  for (auto& it : items) {
    int w = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    bins[w].push_back(it.second);
    load[w] += it.first;
  }
  int k = 0;
  for (int w = 0; w < PL_WARPS; ++w) {
    g.warp_start[w] = (short)k;
    for (int it : bins[w]) g.items[k++] = (unsigned short)it;
  }
  g.warp_start[PL_WARPS] = (short)k;
  // shared memory
  g.sm_goff = (int)align16((size_t)ms * esz);
  g.sm_cb = (int)align16((size_t)g.sm_goff + (size_t)g.E * 8);
  g.sm_tile = (int)align16((size_t)g.sm_cb + (size_t)2 * g.TC * 8);
  size_t tiles = (size_t)2 * g.TC * g.EP * esz;
  if (adjoint) tiles = std::max(tiles, (size_t)g.nslot * PL_RT * PL_RT * esz);  // column-group reduction
  g.smem = (int)(g.sm_tile + tiles);
  if (g.smem > 200 * 1024) return 0;
  *out = g;
  return 1;
}

template <typename K>
static int pl_resident(K k, int smem) {
  int per_sm = 0;
  if ((smem > 48 * 1024 && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, PL_THREADS, smem) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  return per_sm;
}

template <typename CT, int SMAX>
static int pl_resident_t(int adjoint, int smem) {
  return adjoint ? pl_resident(plane_adjoint_kernel<CT, SMAX>, smem) : pl_resident(plane_apply_kernel<CT, SMAX>, smem);
}

template <typename CT>
static int pl_resident_d(int adjoint, int D, int smem) {
  switch (dmax_bucket(D)) {
    case 4: return pl_resident_t<CT, 4>(adjoint, smem);
    case 8: return pl_resident_t<CT, 8>(adjoint, smem);
    case 12: return pl_resident_t<CT, 12>(adjoint, smem);
    case 16: return pl_resident_t<CT, 16>(adjoint, smem);
    case 20: return pl_resident_t<CT, 20>(adjoint, smem);
    default: return pl_resident_t<CT, 24>(adjoint, smem);
  }
}

int plane_preferred(int layout, const AxisView& v) {
  // Two-mode ops on the innermost axis (C = 1): the block-per-CTA kernels
  // read such planes with one sector per lane and re-fetch every sector once
  // per block; the plane kernels read each plane once, coalesced.  Elsewhere
  // the block kernels' direct register loads are already coalesced and
  // cheaper.
  return layout != LAYOUT_DENSE && v.C == 1;
}

int plane_grid(int dtype, const PlaneGeom& g, int adjoint, int nb) {
  // resident CTAs per SM, cached per (device, kernel instance, shared memory)
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int, int>, int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    dev = -1;
  }
  const auto key = std::make_tuple(dev, dtype, dmax_bucket(g.D), adjoint, g.smem);
  int per_sm = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) per_sm = it->second;
  }
  if (!per_sm) {
    per_sm = dtype == FOCK_C64 ? pl_resident_d<float2>(adjoint, g.D, g.smem)
                               : pl_resident_d<double2>(adjoint, g.D, g.smem);
    std::lock_guard<std::mutex> lk(mu);
    cache[key] = per_sm;
  }
  int64_t grid = (int64_t)per_sm * fock_num_sms();
  grid = (grid + nb - 1) / nb;
  if (grid > g.ntiles) grid = g.ntiles;
  if (grid < 1) grid = 1;
  return (int)grid;
}

template <typename CT, int SMAX>
static int pl_launch_t(int adjoint, const void* a, const void* b, void* c, const PlaneGeom& g, int grid,
                       const double2* mat, int mflags, double2* cpart, cudaStream_t st, const BatchArg& bt) {
  if (bt.nb < 1 || bt.nb > 65535) return fock_set_error(FOCK_ERR_INVALID, "batch of %d circuits", bt.nb);
  dim3 gr(grid, 1, bt.nb);
  if (!adjoint) {
    auto k = plane_apply_kernel<CT, SMAX>;
    if (g.smem > 48 * 1024) FOCK_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, g.smem));
    FOCK_CUDA_TRY(launch_kernel(k, gr, dim3(PL_THREADS), g.smem, st, bt.pdl, (const CT*)a, (CT*)c, g, mat, mflags, bt));
  } else {
    auto k = plane_adjoint_kernel<CT, SMAX>;
    if (g.smem > 48 * 1024) FOCK_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, g.smem));
    FOCK_CUDA_TRY(launch_kernel(k, gr, dim3(PL_THREADS), g.smem, st, bt.pdl, (const CT*)a, (const CT*)b, (CT*)c, g, mat,
                                 mflags, cpart, bt));
  }
  return FOCK_OK;
}

template <typename CT>
static int pl_launch_d(int adjoint, const void* a, const void* b, void* c, const PlaneGeom& g, int grid,
                       const double2* mat, int mflags, double2* cpart, cudaStream_t st, const BatchArg& bt) {
  switch (dmax_bucket(g.D)) {
    case 4: return pl_launch_t<CT, 4>(adjoint, a, b, c, g, grid, mat, mflags, cpart, st, bt);
    case 8: return pl_launch_t<CT, 8>(adjoint, a, b, c, g, grid, mat, mflags, cpart, st, bt);
    case 12: return pl_launch_t<CT, 12>(adjoint, a, b, c, g, grid, mat, mflags, cpart, st, bt);
    case 16: return pl_launch_t<CT, 16>(adjoint, a, b, c, g, grid, mat, mflags, cpart, st, bt);
    case 20: return pl_launch_t<CT, 20>(adjoint, a, b, c, g, grid, mat, mflags, cpart, st, bt);
    default: return pl_launch_t<CT, 24>(adjoint, a, b, c, g, grid, mat, mflags, cpart, st, bt);
  }
}

int launch_plane_apply(int dtype, const void* in, void* out, const PlaneGeom& g, int grid, const double2* mat,
                       int mflags, cudaStream_t st, const BatchArg& bt) {
  if (g.ncols <= 0) return FOCK_OK;
  if (dtype == FOCK_C64) return pl_launch_d<float2>(0, in, nullptr, out, g, grid, mat, mflags, nullptr, st, bt);
  return pl_launch_d<double2>(0, in, nullptr, out, g, grid, mat, mflags, nullptr, st, bt);
}

int launch_plane_adjoint(int dtype, const void* psi_in, const void* lam_out, void* lam_in, const PlaneGeom& g,
                         int grid, const double2* mat, int mflags, double2* cpart, cudaStream_t st,
                         const BatchArg& bt) {
  if (dtype == FOCK_C64)
    return pl_launch_d<float2>(1, psi_in, lam_out, lam_in, g, grid, mat, mflags, cpart, st, bt);
  return pl_launch_d<double2>(1, psi_in, lam_out, lam_in, g, grid, mat, mflags, cpart, st, bt);
}
