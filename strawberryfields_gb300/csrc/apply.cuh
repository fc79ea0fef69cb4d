// Strided views of a state tensor for one- and two-axis gates, and the launch
// interface of the apply / adjoint kernels.
#pragma once
#include "gates.cuh"

// Exact division of a 32-bit numerator by a runtime constant d >= 1 as a
// multiply-high and two shifts (round-up multiplier with the add correction:
// m = floor(2^32 (2^l - d) / d) + 1, l = ceil(log2 d);
// q = (t + ((n - t) >> 1)) >> (l - 1) with t = (n * m) >> 32).
struct FastDiv {
  uint32_t d, m;
  int l;
};
inline FastDiv make_fastdiv(uint32_t d) {
  FastDiv f;
  f.d = d;
  f.l = 0;
  while ((1ull << f.l) < d) ++f.l;
  f.m = d == 1 ? 0u : (uint32_t)((((uint64_t)1 << 32) * ((1ull << f.l) - d)) / d + 1);
  return f;
}
__host__ __device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
  if (f.d == 1) return n;
  const uint32_t t = (uint32_t)(((uint64_t)n * f.m) >> 32);
  return (t + ((n - t) >> 1)) >> (f.l - 1);
}

// A gate on axes (ax1 < ax2) of a C-order [D]^naxes tensor sees the state as
// [A][D][B][D][C] (two axes) or [A][D][C] (one axis; B = 1, s2 = 0).
// Column j = (a, b, c), c fastest; element (a, i, b, k, c) sits at
// base(j) + i*s1 + k*s2 with base(j) = a*D*s1 + b*D*s2 + c.
struct AxisView {
  int64_t A, B, C;
  int64_t s1, s2;
  int64_t ncols;
  int fast;         // ncols < 2^32: column indices decomposed by FastDiv
  FastDiv fc, fb;   // division by C and by B
};

AxisView make_view1(int naxes, int D, int ax);
AxisView make_view2(int naxes, int D, int ax1, int ax2);

__device__ __forceinline__ int64_t col_base(const AxisView& v, int64_t j, int D) {
  if (v.fast) {
    const uint32_t jj = (uint32_t)j;
    const uint32_t t = fdiv(jj, v.fc);
    const uint32_t c = jj - t * (uint32_t)v.C;
    const uint32_t a = fdiv(t, v.fb);
    const uint32_t b = t - a * (uint32_t)v.B;
    return (int64_t)a * (v.s1 * D) + (int64_t)b * (v.s2 * D) + c;
  }
  int64_t c = j % v.C;
  int64_t t = j / v.C;
  int64_t b = t % v.B;
  int64_t a = t / v.B;
  return a * (v.s1 * D) + b * (v.s2 * D) + c;
}

// matrix staging flags
#define MF_CONJ 1     // use conj(M)            (bra side of a mixed state)
#define MF_ADJOINT 2  // use M^dagger           (adjoint sweep)
#define MF_SWAP 4     // view axes are (mode2, mode1) of the stored two-mode matrix
#define MF_F32 8      // mat holds complex64 copies of the entries (float2), not double2

// geometry of block b of a view: s entries, offsets base + boff + u*step
struct BlockGeom {
  int s;
  int64_t boff, step;
  int64_t moff;   // offset of the stored block in the matrix
  int rev;        // stored position = s-1-u (swapped SUM blocks)
};

// Grid position y -> block index, largest blocks first (sizes D, D-1, D-1,
// D-2, D-2, ...), so the hardware scheduler starts the longest work first.
__host__ __device__ __forceinline__ int block_of_y(int D, int y) {
  return (D - 1) + ((y & 1) ? -((y + 1) >> 1) : (y >> 1));
}

// Cutoff bucket a kernel instance is compiled for (block sizes 1..DMAX run
// fully unrolled from registers; 0 = generic loop kernel for larger cutoffs).
__host__ __device__ __forceinline__ int dmax_bucket(int D) {
  return D <= 4 ? 4 : D <= 8 ? 8 : D <= 12 ? 12 : D <= 16 ? 16 : D <= 20 ? 20 : D <= 24 ? 24 : 0;
}

__device__ __forceinline__ BlockGeom block_geom(const AxisView& v, int D, int layout, int b, int swap) {
  BlockGeom g;
  if (layout == LAYOUT_DENSE) {
    g.s = D; g.boff = 0; g.step = v.s1; g.moff = 0; g.rev = 0;
    return g;
  }
  g.s = blk_size(D, b);
  if (layout == LAYOUT_SUM) {
    int lo = blk_lo(D, 1, b);
    g.boff = (int64_t)lo * v.s1 + (int64_t)(b - lo) * v.s2;
    g.step = v.s1 - v.s2;
    g.moff = blk_offset(D, b);
    g.rev = swap;
  } else {
    int delta = b - (D - 1);
    int lo = delta > 0 ? delta : 0;
    g.boff = (int64_t)lo * v.s1 + (int64_t)(lo - delta) * v.s2;
    g.step = v.s1 + v.s2;
    int bs = swap ? (2 * D - 2 - b) : b;
    g.moff = blk_offset(D, bs);
    g.rev = 0;
  }
  return g;
}

// Row stride of a staged s x s block: complex64 rows are padded to an even
// length, so one 16-byte shared load carries two entries (row_mac).
template <typename CT>
__host__ __device__ __forceinline__ int ms_stride(int s) {
  return sizeof(CT) == 8 ? (s + 1) & ~1 : s;
}

// Block sizes s run in the unrolled body of size S = s rounded up to a
// multiple of FOCK_S_STEP (columns padded with zeros, rows beyond s
// skipped): a quarter of the bodies per kernel (2.5x smaller objects, faster
// builds) for the same measured speed as one body per size on GB300 (QNN
// gradient 7.40 vs 7.43 ms, single-gate kernels at 12^7 within 3%).
#ifndef FOCK_S_STEP
#define FOCK_S_STEP 4
#endif
static constexpr int kSStep = FOCK_S_STEP;

// state-type slots the staged block of a cutoff-D op needs (s rows at the
// padded row stride)
__host__ __device__ __forceinline__ size_t ms_slots(int, int D) {
  return (size_t)D * ((D + kSStep - 1) / kSStep * kSStep + 2);
}

// Matrix entry idx (FP64, or the complex64 copy with MF_F32) in the state
// precision, conjugated when cj; and the batch offset of a matrix pointer.
template <typename CT>
__device__ __forceinline__ CT mat_entry(const double2* mat, int64_t idx, int cj, int mflags) {
  if (sizeof(CT) == 8 && (mflags & MF_F32)) {
    float2 m = reinterpret_cast<const float2*>(mat)[idx];
    if (cj) m.y = -m.y;
    CT v;
    v.x = m.x;
    v.y = m.y;
    return v;
  }
  double2 m = mat[idx];
  if (cj) m.y = -m.y;
  return to_c(m, (CT*)nullptr);
}
__device__ __forceinline__ const double2* mat_batch(const double2* mat, int64_t entries, int mflags) {
  if (mflags & MF_F32) return reinterpret_cast<const double2*>(reinterpret_cast<const float2*>(mat) + entries);
  return mat + entries;
}

// Stage the s x s block for this CTA into shared memory in the state precision,
// as the matrix that maps the view's input positions to its output positions
// (row w at Ms + w * ms_stride(s)).
template <typename CT>
__device__ __forceinline__ void stage_block(CT* Ms, const double2* mat, const BlockGeom& g, int mflags) {
  const int s = g.s, sp = ms_stride<CT>(s);
  for (int e = threadIdx.x; e < s * s; e += blockDim.x) {
    int w = e / s, u = e - w * s;  // view output w, view input u
    int a = w, c = u;
    if (mflags & MF_ADJOINT) { a = u; c = w; }  // (M^dag)[w][u] = conj(M[u][w])
    if (g.rev) { a = s - 1 - a; c = s - 1 - c; }
    const int cj = ((mflags & MF_ADJOINT) ? 1 : 0) ^ ((mflags & MF_CONJ) ? 1 : 0);
    Ms[w * sp + u] = mat_entry<CT>(mat, g.moff + (int64_t)a * s + c, cj, mflags);
  }
}

// The block for a body of size S >= s: rows w < s at stride ms_stride(S),
// entries u in [s, S) zero.
template <typename CT, int S>
__device__ __forceinline__ void stage_block_pad(CT* Ms, const double2* mat, const BlockGeom& g, int mflags) {
  const int s = g.s, sp = ms_stride<CT>(S);
  const int cj = ((mflags & MF_ADJOINT) ? 1 : 0) ^ ((mflags & MF_CONJ) ? 1 : 0);
  for (int e = threadIdx.x; e < s * S; e += blockDim.x) {
    const int w = e / S, u = e - w * S;
    CT v = czero<CT>();
    if (u < s) {
      int a = w, c = u;
      if (mflags & MF_ADJOINT) { a = u; c = w; }
      if (g.rev) { a = s - 1 - a; c = s - 1 - c; }
      v = mat_entry<CT>(mat, g.moff + (int64_t)a * s + c, cj, mflags);
    }
    Ms[w * sp + u] = v;
  }
}

// A column of s values held in registers in the form the row products use.
// complex64: each value x as the pairs (Re x, Re x) and (Im x, Im x), so a
// row product is two paired FMAs per entry with the staged entry (Re m, Im m)
// as the other operand -- P += m * Re x, Q += m * Im x, and
// m x = (P.re - Q.im, P.im + Q.re) -- half the FP32 instructions of the scalar
// complex FMA; the pairs are built once per column and reused by all s rows.
// (Measured on GB300 against the scalar form and against expanding the staged
// entries instead, which doubles the shared-memory loads: the dense apply at
// 12^7 went from 106 to 96 us and the last-pair beamsplitter from 199 to
// 154 us, the 6-mode cutoff-12 QNN gradient from 8.09 to 7.63 ms.)
template <typename CT, int S> struct ColRegs;
template <int S> struct ColRegs<double2, S> {
  double2 x[S];
  __device__ __forceinline__ void set(const double2 (&v)[S]) {
#pragma unroll
    for (int u = 0; u < S; ++u) x[u] = v[u];
  }
};
template <int S> struct ColRegs<float2, S> {
  f32x2 re[S], im[S];
  __device__ __forceinline__ void set(const float2 (&v)[S]) {
#pragma unroll
    for (int u = 0; u < S; ++u) {
      re[u] = pk2(v[u].x, v[u].x);
      im[u] = pk2(v[u].y, v[u].y);
    }
  }
};

// a += sum_u row[u] x[u] over one staged row (16-byte loads of entry pairs
// for complex64; rows start on 16-byte boundaries)
template <int S>
__device__ __forceinline__ void row_mac(float2& a, const float2* row, const ColRegs<float2, S>& x) {
  const ulonglong2* r2 = reinterpret_cast<const ulonglong2*>(row);
  f32x2 P = 0ull, Q = 0ull;
#pragma unroll
  for (int u2 = 0; u2 < (S + 1) / 2; ++u2) {
    const ulonglong2 m = r2[u2];
    P = ffma2(m.x, x.re[2 * u2], P);
    Q = ffma2(m.x, x.im[2 * u2], Q);
    if (2 * u2 + 1 < S) {
      P = ffma2(m.y, x.re[2 * u2 + 1], P);
      Q = ffma2(m.y, x.im[2 * u2 + 1], Q);
    }
  }
  const float2 p = upk2(P), q = upk2(Q);
  a.x += p.x - q.y;
  a.y += p.y + q.x;
}
template <int S>
__device__ __forceinline__ void row_mac(double2& a, const double2* row, const ColRegs<double2, S>& x) {
#pragma unroll
  for (int u = 0; u < S; ++u) cfma(a, row[u], x.x[u]);
}

// A batch of nb independent circuits of one structure: grid.z indexes the
// circuit; its state, matrix and partial sums sit at z times these strides
// (elements of the state type, double2 entries, double2 entries).
struct BatchArg {
  int nb = 1;
  int64_t state_stride = 0;
  int64_t mat_stride = 0;
  int64_t part_stride = 0;
  int pdl = 0;  // host only: launch with programmatic dependent launch
};

// Programmatic dependent launch.  A kernel launched with the attribute may
// start while its stream predecessor is still running: it does its index
// set-up, then waits in pdl_wait() until the predecessor has completed and
// its writes are visible, before it reads or writes any state, and calls
// pdl_launch_dependents() so that its own successor can be launched once all
// of its CTAs are resident.  Without the attribute both are no-ops.  Because
// every kernel waits for its predecessor's completion, all earlier kernels
// of the stream have completed when the wait returns.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}
template <typename... KArgs, typename... Args>
inline cudaError_t launch_kernel(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, int pdl,
                                 Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k, args...);
}

// Apply a built matrix (FP64 in `mat`, layout LAYOUT_*) on a view: out = M in.
int launch_apply(int dtype, const void* in, void* out, const AxisView& v, int D, int layout,
                 const double2* mat, int mflags, cudaStream_t st, const BatchArg& bt = BatchArg());

// Adjoint step of one op: lam_in = M^dagger lam_out (skipped when lam_in is
// null) and the per-CTA partial sums of
// C[u][v] = sum over columns conj(lam_out[u]) psi_in[v] (stored-matrix
// orientation, FP64).  CTA schedule of one launch: view block y gets gx[y]
// CTAs (the same number for every block), CTAs start[y] .. start[y+1]-1;
// the partial sums of stored block bs sit at part_off[bs] + x * s^2 (x < gx),
// summed in a fixed order by launch_reduce_sched or launch_reduce_ops.
// one entry per photon-number block: 2D - 1 blocks at the largest cutoff
#define ADJ_MAX_BLOCKS (2 * FOCK_MAX_CUTOFF - 1)
struct AdjSched {
  int nblk;
  int total;
  // CTA order: 0 -> block by block (CTA x serves block y for
  // start[y] <= x < start[y+1]); 1 -> interleaved, CTA x serves block
  // x % nblk with rank x / nblk (every block has gx[0] CTAs), so the CTAs of
  // all blocks that read the same columns run together
  int interleave;
  int64_t part_entries;
  int gx[ADJ_MAX_BLOCKS];
  int start[ADJ_MAX_BLOCKS + 1];
  int64_t part_off[ADJ_MAX_BLOCKS];
};
// nb: circuits of a batch launched together (grid.z); ctas_per_sm: CTAs per
// SM the launch spreads over all blocks and circuits (the default measured
// best for the 6-mode cutoff-12 QNN; fock_plan_tune changes it per op)
AdjSched make_adj_sched(int dtype, const AxisView& v, int D, int layout, int nb = 1, int ctas_per_sm = 8);
// two-mode ops on the innermost axis pair (C = 1) run their block CTAs
// interleaved: each block reads a few elements of every sector of the
// columns' planes, so the blocks that share a plane should read it together
// (from L2) rather than one block after another (from DRAM)
__host__ __device__ __forceinline__ int interleave_blocks(int layout, const AxisView& v) {
  return layout != LAYOUT_DENSE && v.C == 1;
}
int launch_adjoint_partials(int dtype, const void* psi_in, const void* lam_out, void* lam_in,
                            const AxisView& v, int D, int layout, const double2* mat, int mflags,
                            double2* cpart, const AdjSched& sc, cudaStream_t st, const BatchArg& bt = BatchArg());
int launch_reduce_partials(const double2* cpart, int gx, int64_t nent, double2* cout, cudaStream_t st, int nb = 1,
                           int64_t part_stride = 0, int64_t out_stride = 0, int pdl = 0);
// All ops' partials in one launch: op k's partials sit at cpart_off; entry e
// of its C (stored orientation) is the fixed-order sum over x < gx of
// cpart[cpart_off + x * nent + e] (plane layout) or of
// cpart[cpart_off + gx * blk_offset(bs) + x * s^2 + e_in_block] (block
// schedules, one gx for every block).
struct RedOp {
  int64_t c_off, cpart_off;
  int nent, gx, plane, layout;
  int chunk0;  // first reduction CTA of this op
  int ec;      // C entries per reduction CTA: 32, 16 or 8 (more partial rows, fewer entries)
};
#define RED_THREADS 256
// entries per reduction CTA for an op with gx partial rows: the CTA's
// RED_THREADS / ec row segments keep each thread's serial sum short
__host__ __device__ __forceinline__ int red_entries_per_cta(int gx) { return gx <= 128 ? 32 : gx <= 512 ? 16 : 8; }
int launch_reduce_ops(const RedOp* ops, int n_ops, int64_t chunks, int D, const double2* cpart, double2* carena,
                      cudaStream_t st, int nb, int64_t part_stride, int64_t out_stride);
// sum the partials of a schedule into `cout` (stored orientation, layout entries)
int launch_reduce_sched(const double2* cpart, const AdjSched& sc, int D, int layout, double2* cout, cudaStream_t st,
                        int nb = 1, int64_t part_stride = 0, int64_t out_stride = 0, int pdl = 0);

// Plane-tile kernels (plane.cu): a persistent CTA stages TC columns' whole
// planes (D elements for one mode, D x D for two) in shared memory and applies
// every block of the op to them.  The geometry is built once per op on the
// host and passed by value.
#define PL_THREADS 256
#define PL_WARPS 8
#define PL_MAX_BLK 48
#define PL_MAX_ITEMS 128
#define PL_RT 3            // C pass: each thread sums a PL_RT x PL_RT sub-block of one block's C
#define PL_MAX_CITEMS 384  // C sub-blocks of the largest plane (366 at cutoff 16)
#define PL_MAX_D1 24  // one-mode ops up to this cutoff
#define PL_MAX_D2 16  // two-mode ops up to this cutoff (D*D <= PL_THREADS rows)
struct PlaneGeom {
  int64_t A, B, C, s1, s2, ncols, ntiles;  // view [A][D][B][D][C] and its columns
  int D, E, EP, TC;       // cutoff, plane elements, padded row, columns per tile
  int two, c_inner;       // two-mode plane; copy with lanes over columns
  int flat;               // plane of column j starts at j*E (gate on the innermost axes)
  unsigned emagic;        // ceil(2^26 / E): idx / E as a multiply-shift
  int nblk, G, nslot;     // blocks; column groups and (sub-block, group) slots of the C pass
  int ncitems;            // C sub-blocks (PL_RT x PL_RT)
  int nent, ms_total;     // C entries (= staged matrix entries)
  int sm_goff, sm_cb, sm_tile, smem;  // shared-memory layout (bytes)
  short base[PL_MAX_BLK], step[PL_MAX_BLK], s[PL_MAX_BLK];  // block y: elements base + u*step
  int ms_off[PL_MAX_BLK + 1];  // staged matrix of block y (prefix of s^2)
  int moff[PL_MAX_BLK];        // stored matrix offset of block y
  int cout_off[PL_MAX_BLK];    // offset of block y's C entries (stored orientation)
  unsigned char rev[PL_MAX_BLK];
  short warp_start[PL_WARPS + 1];
  unsigned short items[PL_MAX_ITEMS];  // (block << 4) | column group, per warp
  unsigned short citems[PL_MAX_CITEMS];  // (block << 10) | (row0 << 5) | col0 of each C sub-block
};
// 0 when the op does not fit the plane kernels (then the block kernels run)
// tile_columns: columns per tile of a two-mode plane op (0: 32)
int make_plane_geom(int dtype, const AxisView& v, int D, int layout, int swap, int adjoint, PlaneGeom* g,
                    int tile_columns = 0);
int plane_grid(int dtype, const PlaneGeom& g, int adjoint, int nb);
// the ops the plane kernels run by default (the others keep the block kernels)
int plane_preferred(int layout, const AxisView& v);
int launch_plane_apply(int dtype, const void* in, void* out, const PlaneGeom& g, int grid, const double2* mat,
                       int mflags, cudaStream_t st, const BatchArg& bt = BatchArg());
// lam_in = M^dagger lam_out (skipped when lam_in is null) and per-CTA partial
// C sums in cpart[grid][g.nent]; reduce with launch_reduce_partials(gx = grid)
int launch_plane_adjoint(int dtype, const void* psi_in, const void* lam_out, void* lam_in, const PlaneGeom& g,
                         int grid, const double2* mat, int mflags, double2* cpart, cudaStream_t st,
                         const BatchArg& bt = BatchArg());

// slot of op j's output in a forward sweep that keeps every k-th state
// (k = store_every): 0 -> ping-pong slots 0/1; 1 -> slot j; k > 1 -> the
// checkpoint slot (j+1)/k - 1 when (j+1) % k == 0 or j is the last op,
// otherwise one of two scratch slots after the n_ckpt checkpoints.
__host__ __device__ __forceinline__ int64_t out_slot(int j, int n_ops, int k) {
  if (k <= 0) return j & 1;
  if (k == 1) return j;
  const int64_t nc = (n_ops + k - 1) / k;
  if ((j + 1) % k == 0) return (j + 1) / k - 1;
  if (j == n_ops - 1) return nc - 1;
  return nc + (j & 1);
}

// Persistent sweeps (sweep.cu): one cooperative launch walks every op of a
// plan, all CTAs meeting at a grid barrier between ops.  For states small
// enough that per-launch ramp and tail cost more than the op itself.
struct SweepOp {
  AxisView view;
  int layout, mflags;
  int64_t m_off;      // matrix in the arena (double2 entries)
  int64_t c_off;      // the op's C entries in the C arena
  int64_t part_base;  // the op's partial sums (double2 entries)
  int nent;           // C entries
  int fwd_nx;         // column tiles per block in the forward sweep
  AdjSched sc;        // adjoint CTA schedule; sc.total <= grid
};
// grid-barrier state in device memory: arrival count, generation, error
// flag, and one item counter per op (all zero at launch)
struct SweepSync {
  unsigned* count;
  unsigned* gen;
  int* err;
  unsigned* items;
  unsigned spin_limit;  // polls of the generation word before a barrier gives up
};
#define SWEEP_SPIN_LIMIT_DEFAULT (1u << 24)
// CTAs per launch that can be co-resident (0: no persistent kernel for D)
int sweep_grid(int dtype, int D, int backward);
// adjoint schedule for a persistent sweep: every block's CTAs fit in `grid`
AdjSched make_adj_sched_grid(int dtype, const AxisView& v, int D, int layout, int grid);
int launch_sweep_forward(int dtype, int D, const SweepOp* ops, int n_ops, int store_every, const void* state_in,
                         void* states, int64_t slot_elems, const double2* arena, SweepSync sync, int grid,
                         cudaStream_t st);
int launch_sweep_backward(int dtype, int D, const SweepOp* ops, int n_ops, const void* state_in, const void* states,
                          int64_t slot_elems, void* lam_a, void* lam_b, const double2* arena, double2* cpart,
                          double2* carena, int64_t carena_entries, SweepSync sync, int grid, cudaStream_t st);

// Fused op groups of the forward sweep on a three-mode tile (tile.cu): pure
// complex64 states, cutoff <= 16.  Tile axes 0 < 1 < 2 are the group's modes
// in increasing order; the other modes index the columns.
#define TL_THREADS 256
#define TL_MAX_OPS 16
#define TL_MAX_REST 32
struct TileOp {
  int layout;          // LAYOUT_DENSE / SUM / DIFF
  int ta, tb;          // tile axes (ta < tb; tb = -1 for one-mode ops)
  int swap;            // stored matrix orientation is (tb, ta)
  int64_t m_off;       // matrix in the arena
  int64_t store_slot;  // slot that receives this op's output (-1: none)
};
struct TileGroupArg {
  int D, T, nops, nrest, TC, lgTC, c_fast;
  int64_t S[3];                      // global strides of the tile modes
  int64_t rest_stride[TL_MAX_REST];  // global strides of the other modes, slowest first
  int64_t ncols, nchunks;            // columns, chunks of TC columns
  int64_t slot_elems;                // elements of one stored-state slot (whole batch)
  TileOp ops[TL_MAX_OPS];
};
size_t tile_smem_bytes(int D, int TC);
int launch_tile_forward(const TileGroupArg& g, const void* in, void* states, const double2* arena, int grid,
                        cudaStream_t st, const BatchArg& bt);

// reduced density matrix pieces (capi.cu)
int launch_rdm_mixed(int dtype, const void* state, int num_modes, int D, int mode, int64_t ntr, int chunks,
                     double2* part, cudaStream_t st);
int launch_transpose_dm(const double2* C, double2* out, int D, cudaStream_t st);
int check_reduced_dm1_args(int num_modes, int cutoff, int pure, int dtype, int mode, const void* state,
                           const void* out);

// single matrix build with inline parameters (gates.cu)
int build_single(int gate, int layout, int D, double p0, double p1, const PhaseTerm* terms,
                 int nterm, double2* M, double2* dM, double2* scratch, cudaStream_t st);
