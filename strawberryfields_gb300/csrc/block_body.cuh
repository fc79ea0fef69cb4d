// Device bodies of the block-per-CTA kernels, shared by the one-op-per-launch
// kernels (apply.cu, adjoint.cu) and the persistent sweep kernels (sweep.cu).
//
// Apply: each thread takes one column of one photon-number block (or of the
// dense single-mode block): it loads the s values into registers, multiplies
// by the s x s block staged in shared memory and stores s outputs.
// Adjoint: a CTA stages TILE columns of lam_out and psi_in in shared memory
// (cp.async), forms lam_in = M^dagger lam_out per column and accumulates
// C = sum_columns conj(lam_out) psi_in^T as a register-tiled GEMM.
#pragma once
#include "apply.cuh"

#define APPLY_THREADS 256
#define APPLY_COLS 1

// State loads: through the read-only (non-coherent) path when the input is
// not written during the launch (one op per launch); as ordinary loads (COH)
// when other CTAs of the same persistent launch wrote it -- those are
// coherent after the grid barrier's acquire fence and keep the L1 sector
// reuse of the gates on the innermost axes.
template <bool COH, typename CT>
__device__ __forceinline__ CT ld_state(const CT* p) {
  if (COH) return *p;
  return __ldg(p);
}

// The column's loads are issued before the block is staged in shared memory,
// so the two global round trips overlap.
// staged: the block is in shared memory already (the kernel staged it before
// waiting for its stream predecessor)
template <typename CT, int S, bool COH>
__device__ __forceinline__ void apply_cols(const CT* __restrict__ in, CT* __restrict__ out,
                                           const AxisView& v, int D, CT* Ms, const double2* mat, int mflags,
                                           const BlockGeom& g, int64_t j0, int staged) {
  const bool valid = j0 < v.ncols;
  const int s = g.s;  // <= S
  const int64_t b0 = valid ? col_base(v, j0, D) + g.boff : 0;
  CT x0[S];
  // complex64 column contiguous in memory (a one-mode op on the innermost
  // axis) with an even length on a 16-byte boundary (checked on the
  // addresses: a state may start at any 8-byte offset): 16-byte loads and
  // stores of element pairs, half the memory instructions
  const bool pairs = sizeof(CT) == 8 && g.step == 1 && !(s & 1) &&
                     !(((uintptr_t)(in + b0) | (uintptr_t)(out + b0)) & 15);
  if (valid) {
    if constexpr (sizeof(CT) == 8) {
      if (pairs) {
        const float4* p4 = reinterpret_cast<const float4*>(in + b0);
#pragma unroll
        for (int u2 = 0; u2 < S / 2; ++u2) {
          const float4 q = 2 * u2 < s ? ld_state<COH>(p4 + u2) : make_float4(0.f, 0.f, 0.f, 0.f);
          x0[2 * u2] = CT{q.x, q.y};
          x0[2 * u2 + 1] = CT{q.z, q.w};
        }
      }
    }
    if (!pairs) {
#pragma unroll
      for (int u = 0; u < S; ++u) x0[u] = u < s ? ld_state<COH>(in + b0 + u * g.step) : czero<CT>();
    }
  }
  if (!staged) stage_block_pad<CT, S>(Ms, mat, g, mflags);
  __syncthreads();
  if (!valid) return;
  constexpr int SP = sizeof(CT) == 8 ? (S + 1) & ~1 : S;
  ColRegs<CT, S> xc;
  xc.set(x0);
  // rows one at a time: unrolled, the loads of later rows run ahead and
  // spill the column's registers
  if constexpr (sizeof(CT) == 8) {
    if (pairs) {
#pragma unroll 1
      for (int w = 0; w < s; w += 2) {
        CT a0 = czero<CT>(), a1 = czero<CT>();
        row_mac<S>(a0, Ms + w * SP, xc);
        row_mac<S>(a1, Ms + (w + 1) * SP, xc);
        *reinterpret_cast<float4*>(out + b0 + w) = make_float4(a0.x, a0.y, a1.x, a1.y);
      }
      return;
    }
  }
#pragma unroll 1
  for (int w = 0; w < s; ++w) {
    CT a0 = czero<CT>();
    row_mac<S>(a0, Ms + w * SP, xc);
    out[b0 + w * g.step] = a0;
  }
}

template <typename CT, bool COH>
__device__ void apply_cols_generic(const CT* __restrict__ in, CT* __restrict__ out, const AxisView& v,
                                   int D, CT* Ms, const double2* mat, int mflags, const BlockGeom& g,
                                   int64_t j0, int staged) {
  if (!staged) stage_block(Ms, mat, g, mflags);
  __syncthreads();
  for (int k = 0; k < APPLY_COLS; ++k) {
    const int64_t j = j0 + k * APPLY_THREADS;
    if (j >= v.ncols) break;
    const int64_t base = col_base(v, j, D) + g.boff;
    const int S = g.s, SP = ms_stride<CT>(S);
    for (int w = 0; w < S; ++w) {
      CT acc = czero<CT>();
      for (int u = 0; u < S; ++u) cfma(acc, Ms[w * SP + u], ld_state<COH>(in + base + u * g.step));
      out[base + w * g.step] = acc;
    }
  }
}

// s <= S ? run the unrolled body of size S : try S + kSStep (up to DMAX)
template <typename CT, int S, int DMAX, bool COH = false>
struct ApplyDispatch {
  __device__ __forceinline__ static void run(const CT* in, CT* out, const AxisView& v, int D, CT* Ms,
                                             const double2* mat, int mflags, const BlockGeom& g, int64_t j0,
                                             int staged = 0) {
    if (g.s <= S) apply_cols<CT, S, COH>(in, out, v, D, Ms, mat, mflags, g, j0, staged);
    else ApplyDispatch<CT, S + kSStep, DMAX, COH>::run(in, out, v, D, Ms, mat, mflags, g, j0, staged);
  }
};
template <typename CT, int DMAX, bool COH>
struct ApplyDispatch<CT, DMAX + kSStep, DMAX, COH> {
  __device__ __forceinline__ static void run(const CT* in, CT* out, const AxisView& v, int D, CT* Ms,
                                             const double2* mat, int mflags, const BlockGeom& g, int64_t j0,
                                             int staged = 0) {
    apply_cols_generic<CT, COH>(in, out, v, D, Ms, mat, mflags, g, j0, staged);
  }
};

// The block staged as the body of size S >= s that the dispatch above picks
// (the layout apply_cols / adjoint_body read), or as the generic loop's block.
template <typename CT, int S, int DMAX>
struct StageDispatch {
  __device__ __forceinline__ static void run(CT* Ms, const double2* mat, const BlockGeom& g, int mflags) {
    if (g.s <= S) stage_block_pad<CT, S>(Ms, mat, g, mflags);
    else StageDispatch<CT, S + kSStep, DMAX>::run(Ms, mat, g, mflags);
  }
};
template <typename CT, int DMAX>
struct StageDispatch<CT, DMAX + kSStep, DMAX> {
  __device__ __forceinline__ static void run(CT* Ms, const double2* mat, const BlockGeom& g, int mflags) {
    stage_block(Ms, mat, g, mflags);
  }
};

// resident CTAs per SM the register budget allows: 4 (32 warps) up to cutoff
// 12, 3 up to 20 (the batched workload's bulk), 2 beyond
template <int DMAX> struct ApplyMinBlocks { static const int value = (DMAX > 0 && DMAX <= 12) ? 4 : (DMAX > 0 && DMAX <= 20) ? 3 : 2; };


template <int S> struct RRof { static const int value = (S + 3) / 4; };

// Asynchronous global -> shared copies (cp.async): the tile lands in shared
// memory without passing through registers; invalid columns are zero-filled.
__device__ __forceinline__ void cp_async_elem(float2* dst, const float2* src, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(src), "r"(valid ? 8 : 0));
}
__device__ __forceinline__ void cp_async_elem(double2* dst, const double2* src, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(src), "r"(valid ? 16 : 0));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_group1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

template <typename CT, int S, int TILE>
__device__ __forceinline__ void adjoint_body(const CT* __restrict__ psi_in, const CT* __restrict__ lam_out,
                                             CT* __restrict__ lam_in, const AxisView& v, int D, CT* MsH,
                                             const double2* __restrict__ mat, int mflags, CT* lam_s, CT* psi_s,
                                             const BlockGeom& g, double2* __restrict__ mypart, int xrank, int gxb,
                                             int write_lam, int staged) {
  constexpr int RR = RRof<S>::value;
  constexpr int NG = TILE / 16;
  constexpr int LD = TILE + 1;  // padded row stride (elements)
  const int tid = threadIdx.x;
  const int s = g.s;  // <= S
  const int owner = tid / NG, grp = tid - owner * NG;
  const int ro = owner >> 2, co = owner & 3;
  CT acc[RR][RR];
#pragma unroll
  for (int r = 0; r < RR; ++r)
#pragma unroll
    for (int c = 0; c < RR; ++c) acc[r][c] = czero<CT>();

  const int64_t ntiles = (v.ncols + TILE - 1) / TILE;
  int64_t tile_base = 0;  // this thread's column base in the last issued tile
  auto issue = [&](int64_t t) {
    const int64_t j = t * TILE + tid;
    const bool valid = j < v.ncols;
    const int64_t base = valid ? col_base(v, j, D) + g.boff : 0;
    tile_base = base;
    // two groups: lam_out (L2-resident, needed first for lam_in), then psi_in
#pragma unroll
    for (int u = 0; u < S; ++u) {
      const bool vu = valid && u < s;  // rows s..S-1 zero-filled
      const int64_t off = vu ? base + u * g.step : 0;
      cp_async_elem(&lam_s[u * LD + tid], lam_out + off, vu);
    }
    cp_async_commit();
#pragma unroll
    for (int u = 0; u < S; ++u) {
      const bool vu = valid && u < s;
      const int64_t off = vu ? base + u * g.step : 0;
      cp_async_elem(&psi_s[u * LD + tid], psi_in + off, vu);
    }
    cp_async_commit();
  };
  // the first tile's copies are in flight while the block is staged
  if (xrank < ntiles) issue(xrank);
  if (write_lam && !staged) stage_block_pad<CT, S>(MsH, mat, g, mflags | MF_ADJOINT);
  // padding rows S..4*RR-1 stay zero
  for (int e = tid; e < (4 * RR - S) * LD; e += TILE) {
    lam_s[S * LD + e] = czero<CT>();
    psi_s[S * LD + e] = czero<CT>();
  }
  __syncthreads();
  for (int64_t t = xrank; t < ntiles; t += gxb) {
    cp_async_wait_group1();  // this thread's lam_out column has landed
    const int64_t j = t * TILE + tid;
    if (write_lam && j < v.ncols) {
      // each thread reads back only its own column: no barrier needed here
      const int64_t base = tile_base;
      constexpr int SP = sizeof(CT) == 8 ? (S + 1) & ~1 : S;
      CT lam[S];
#pragma unroll
      for (int u = 0; u < S; ++u) lam[u] = lam_s[u * LD + tid];
      ColRegs<CT, S> lc;
      lc.set(lam);
      // two rows per pass: four independent FMA chains instead of two
      int w = 0;
#pragma unroll 1
      for (; w + 1 < s; w += 2) {
        CT a0 = czero<CT>(), a1 = czero<CT>();
        row_mac<S>(a0, MsH + w * SP, lc);
        row_mac<S>(a1, MsH + (w + 1) * SP, lc);
        lam_in[base + w * g.step] = a0;
        lam_in[base + (w + 1) * g.step] = a1;
      }
      if (w < s) {
        CT a = czero<CT>();
        row_mac<S>(a, MsH + w * SP, lc);
        lam_in[base + w * g.step] = a;
      }
    }
    cp_async_wait_all();  // and its psi_in column
    __syncthreads();  // every thread's column of tile t has landed
#pragma unroll 4
    for (int step = 0; step < TILE / NG; ++step) {
      const int col = step * NG + grp;
      CT lv[RR], pv[RR];
#pragma unroll
      for (int r = 0; r < RR; ++r) lv[r] = lam_s[(ro * RR + r) * LD + col];
#pragma unroll
      for (int c = 0; c < RR; ++c) pv[c] = psi_s[(co * RR + c) * LD + col];
#pragma unroll
      for (int r = 0; r < RR; ++r)
#pragma unroll
        for (int c = 0; c < RR; ++c) cfma_conj(acc[r][c], lv[r], pv[c]);
    }
    __syncthreads();  // the tile buffers are free for the next tile
    if (t + gxb < ntiles) issue(t + gxb);
  }
  // reduce over the NG groups of each owner (adjacent lanes)
#pragma unroll
  for (int off = NG / 2; off > 0; off >>= 1) {
#pragma unroll
    for (int r = 0; r < RR; ++r)
#pragma unroll
      for (int c = 0; c < RR; ++c) {
        acc[r][c].x += __shfl_xor_sync(0xffffffffu, acc[r][c].x, off);
        acc[r][c].y += __shfl_xor_sync(0xffffffffu, acc[r][c].y, off);
      }
  }
  if (grp == 0) {
#pragma unroll
    for (int r = 0; r < RR; ++r)
#pragma unroll
      for (int c = 0; c < RR; ++c) {
        int u = ro * RR + r, w = co * RR + c;
        if (u < s && w < s) {
          int a = g.rev ? s - 1 - u : u;
          int b = g.rev ? s - 1 - w : w;
          mypart[a * s + b] = to_d(acc[r][c]);
        }
      }
  }
}

template <typename CT, int TILE>
__device__ void adjoint_generic(const CT* __restrict__ psi_in, const CT* __restrict__ lam_out,
                                CT* __restrict__ lam_in, const AxisView& v, int D, CT* MsH,
                                const double2* __restrict__ mat, int mflags, const BlockGeom& g,
                                double2* __restrict__ mypart, int xrank, int gxb, int write_lam, int staged) {
  if (write_lam && !staged) stage_block(MsH, mat, g, mflags | MF_ADJOINT);
  __syncthreads();
  // large blocks (beyond the unrolled buckets): thread per C entry over this
  // CTA's share of the columns, then lam_in per column
  const int S = g.s;
  const int64_t per = (v.ncols + gxb - 1) / gxb;
  int64_t j0 = xrank * per, j1 = j0 + per;
  if (j1 > v.ncols) j1 = v.ncols;
  for (int e = threadIdx.x; e < S * S; e += blockDim.x) {
    int u = e / S, w = e - u * S;
    double2 a = make_double2(0.0, 0.0);
    for (int64_t j = j0; j < j1; ++j) {
      const int64_t base = col_base(v, j, D) + g.boff;
      double2 ld = to_d(lam_out[base + u * g.step]), pd = to_d(psi_in[base + w * g.step]);
      cfma_conj(a, ld, pd);
    }
    int aa = g.rev ? S - 1 - u : u, bb = g.rev ? S - 1 - w : w;
    mypart[aa * S + bb] = a;
  }
  if (!write_lam) return;
  for (int64_t j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    const int64_t base = col_base(v, j, D) + g.boff;
    const int SP = ms_stride<CT>(S);
    for (int w = 0; w < S; ++w) {
      CT a = czero<CT>();
      for (int u = 0; u < S; ++u) cfma(a, MsH[w * SP + u], lam_out[base + u * g.step]);
      lam_in[base + w * g.step] = a;
    }
  }
}

template <typename CT, int S, int DMAX, int TILE>
struct AdjDispatch {
  __device__ __forceinline__ static void run(const CT* psi_in, const CT* lam_out, CT* lam_in, const AxisView& v,
                                             int D, CT* MsH, const double2* mat, int mflags, CT* lam_s, CT* psi_s,
                                             const BlockGeom& g, double2* mypart, int xrank, int gxb,
                                             int write_lam, int staged = 0) {
    if (g.s <= S)
      adjoint_body<CT, S, TILE>(psi_in, lam_out, lam_in, v, D, MsH, mat, mflags, lam_s, psi_s, g, mypart, xrank,
                                gxb, write_lam, staged);
    else
      AdjDispatch<CT, S + kSStep, DMAX, TILE>::run(psi_in, lam_out, lam_in, v, D, MsH, mat, mflags, lam_s, psi_s,
                                                   g, mypart, xrank, gxb, write_lam, staged);
  }
};
template <typename CT, int DMAX, int TILE>
struct AdjDispatch<CT, DMAX + kSStep, DMAX, TILE> {
  __device__ __forceinline__ static void run(const CT* psi_in, const CT* lam_out, CT* lam_in, const AxisView& v,
                                             int D, CT* MsH, const double2* mat, int mflags, CT*, CT*,
                                             const BlockGeom& g, double2* mypart, int xrank, int gxb,
                                             int write_lam, int staged = 0) {
    adjoint_generic<CT, TILE>(psi_in, lam_out, lam_in, v, D, MsH, mat, mflags, g, mypart, xrank, gxb, write_lam,
                              staged);
  }
};

// register budget of the adjoint: 3 resident CTAs (24 warps) per SM for
// complex64 cutoffs up to 12, 2 up to 20 (a few hundred bytes of spill at 20,
// measured 18% faster on the heterogeneous batch than 1 CTA/SM), else 1
template <typename CT, int DMAX> struct AdjMinBlocks {
  static const int value = (sizeof(CT) == 8 && DMAX > 0 && DMAX <= 12) ? 3 : (sizeof(CT) == 8 && DMAX > 0 && DMAX <= 20) ? 2 : 1;
};

