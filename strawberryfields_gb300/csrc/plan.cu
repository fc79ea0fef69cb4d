// Compiled circuits: gate-list fusion, forward sweep and adjoint sweep.
//
// fock_plan_create compiles a gate list on the host.  Rotation and Kerr gates
// (diagonal in the Fock basis) never get their own pass over the state: they
// become phase terms of the next non-diagonal gate on the same mode (input
// side), or of the last one (output side) when no later gate touches the
// mode; cross-Kerr becomes a phase term of a two-mode gate on the same pair
// or, failing that, its own identity op.  Each remaining op reads and writes
// the state once.  The reference applies every gate as its own pass
// (LocalEngine._run_program, strawberryfields/engine.py:422-471, calling
// Circuit.apply_gate_BLAS / apply_twomode_gate per gate).
//
// Device tables (build jobs, phase terms, gradient contributions) live at the
// head of the caller's workspace and are copied there from pinned host memory
// on every call, so a captured CUDA graph replays them.
#include "apply.cuh"

#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <vector>

namespace {

struct PlanOp {
  int layout = 0;
  int gate = GATE_IDENTITY;
  int mode1 = -1, mode2 = -1;
  int pidx = -1;
  int n_fused = 0;
  // state axes the op acts on (modes for a ket; 2m / 2m+1 for the ket / bra
  // side of a density matrix), bra-side flag, and the op whose matrix it uses
  int axis_a = -1, axis_b = -1;
  int conj = 0;
  int owner = -1;
  std::vector<PhaseTerm> terms;
  std::vector<GradContrib> contribs;  // .op filled at finalize
  // derived
  AxisView view;
  int swap = 0;
  int64_t m_off = 0, dm_off = -1, scratch_off = -1, c_off = 0;
  AdjSched sched;  // CTA schedule and partial-sum layout of the adjoint launch
  int64_t nent = 0;
  // plane-tile kernels (when the op fits them): geometry and persistent grids
  int plane = 0;     // plane-tile kernels selected for this op
  int plane_ok = 0;  // the plane geometry exists (fock_plan_tune may select it)
  PlaneGeom pg_fwd, pg_adj;
  int grid_fwd = 0, grid_adj = 0;
  int adj_ctas = 8;  // adjoint CTAs per SM (block kernels)
  int pl_tc = 0;     // plane-tile columns of a two-mode op (0: the default 32)
  // fused tile group of the forward sweep this op belongs to (-1: none)
  int group = -1;
  // persistent-sweep adjoint schedule and partial-sum region
  AdjSched psched;
  int64_t ppart_off = 0;
  int64_t cpart_off = 0;  // this op's partial-sum region (reduce_at_end)
};

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// matrix staging flags of an op: swapped view axes, bra side (conj M)
inline int op_flags(const PlanOp& op) { return (op.swap ? MF_SWAP : 0) | (op.conj ? MF_CONJ : 0); }

}  // namespace

struct fock_plan {
  int N = 0, D = 0, pure = 1, dtype = 0, n_params = 0, n_gates = 0;
  int n_jobs = 0;  // matrix builds (ops that own a matrix)
  int batch = 1;  // circuits of this structure run together (grid.z)
  std::vector<PlanOp> ops;
  // table image (pinned host memory) and its sections
  unsigned char* host = nullptr;
  size_t tables_bytes = 0;
  size_t o_jobs = 0, o_terms = 0, o_gops = 0, o_contrib = 0, o_pstart = 0, o_plist = 0;
  int n_terms = 0, n_contrib = 0;
  // workspace sections
  size_t o_arena = 0, o_carena = 0, o_cpart = 0, ws_bytes = 0;
  int64_t arena_entries = 0, carena_entries = 0, cpart_entries = 0;
  // partial sums: one region per op, reduced by one launch after the sweep
  // (when they fit the budget), or one shared region reduced after every op
  int reduce_at_end = 0;
  int red_chunks = 0;  // CTAs of the end-of-sweep reduction
  size_t o_red = 0;
  int64_t state_elems = 0;
  int64_t flops_fwd = 0;
  // persistent sweeps (small states): grids, tables, sync words, partials
  int persist = 0;
  int g_fwd = 0, g_bwd = 0;
  unsigned spin_limit = SWEEP_SPIN_LIMIT_DEFAULT;
  // fused three-mode tile groups: ops [k0, k1) on modes m[0] < m[1] < m[2]
  struct Group {
    int k0, k1;
    int m[3];
  };
  std::vector<Group> groups;
  int tile_tc = 0;     // columns per chunk
  int tile_grid = 0;   // CTAs of a forward group launch
  size_t o_sweep = 0, o_sync = 0, o_ppart = 0;
  int64_t ppart_entries = 0;
  // complex64 plans: the sweep kernels stage complex64 copies of the
  // matrices (o_arena32, converted after every build), not the FP64 arena
  int mat32 = 0;
  size_t o_arena32 = 0;
  // optional per-op timing
  int timing = 0;
  std::vector<cudaEvent_t> ev_fwd, ev_bwd;
  int fwd_recorded = 0, bwd_recorded = 0;
};

// Record a timing event; inside a stream capture it must be an external
// event-record node so that elapsed times can be read after each replay.
static int record_event(cudaEvent_t ev, cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  FOCK_CUDA_TRY(cudaStreamIsCapturing(st, &cs));
  if (cs == cudaStreamCaptureStatusActive) FOCK_CUDA_TRY(cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal));
  else FOCK_CUDA_TRY(cudaEventRecord(ev, st));
  return FOCK_OK;
}

static int ensure_events(std::vector<cudaEvent_t>& ev, size_t n) {
  while (ev.size() < n) {
    cudaEvent_t e;
    FOCK_CUDA_TRY(cudaEventCreate(&e));
    ev.push_back(e);
  }
  return FOCK_OK;
}

// ---------------------------------------------------------------------------
// compile
// ---------------------------------------------------------------------------
static int is_diag1(int k) { return k == FOCK_ROTATION || k == FOCK_KERR; }
static int is_two(int k) {
  return k == FOCK_BEAMSPLITTER || k == FOCK_MZGATE || k == FOCK_CROSS_KERR || k == FOCK_TWO_MODE_SQUEEZE;
}

// add a phase term (with its gradient contribution) to op
static void add_term(PlanOp& op, int fn, int side, int pidx, int neg = 0) {
  op.terms.push_back(PhaseTerm{fn, side, pidx, neg, 0.0});
  GradContrib g;
  g.op = -1;
  g.type = side ? GC_W_OUT : GC_W_IN;
  g.fn = fn;
  g.pidx = pidx;
  g.scale = neg ? -1.0 : 1.0;
  op.contribs.push_back(g);
  op.n_fused++;
}

// a phase on mode m of a density matrix, carried by the loss superoperator
// on the (ket, bra) pair: exp(i p f(n_ket)) on the ket axis and
// exp(-i p f(n_bra)) on the bra axis
static void add_loss_terms(PlanOp& op, int fn, int side, int pidx) {
  add_term(op, fn, side, pidx, 0);
  add_term(op, fn == FN_A ? FN_B : FN_B2, side, pidx, 1);
  op.n_fused--;
}

static void add_contrib(PlanOp& op, int type, int fn, int pidx, double scale) {
  GradContrib g;
  g.op = -1;
  g.type = type;
  g.fn = fn;
  g.pidx = pidx;
  g.scale = scale;
  op.contribs.push_back(g);
}

struct Pending {
  int fn;     // FN_A (rotation) or FN_A2 (Kerr) relative to the mode
  int pidx;
};
struct PendingCK {
  int a, b, pidx;
};

// move pending single-mode terms of `mode` into op as input-side terms
static void absorb_pending(PlanOp& op, int mode, std::vector<std::vector<Pending>>& pend) {
  if (op.gate == FOCK_LOSS) {
    for (const Pending& p : pend[mode]) add_loss_terms(op, p.fn, 0, p.pidx);
    pend[mode].clear();
    return;
  }
  const int slot_b = (op.layout != LAYOUT_DENSE && op.mode2 == mode);
  for (const Pending& p : pend[mode]) {
    int fn = p.fn;
    if (slot_b) fn = (fn == FN_A) ? FN_B : FN_B2;
    add_term(op, fn, 0, p.pidx);
  }
  pend[mode].clear();
}

// table of the one-launch reduction (in the pinned table image)
static void write_red_table(fock_plan* P) {
  RedOp* red = (RedOp*)(P->host + P->o_red);
  int chunks = 0;
  for (size_t k = 0; k < P->ops.size(); ++k) {
    const PlanOp& op = P->ops[k];
    red[k].c_off = op.c_off;
    red[k].cpart_off = op.cpart_off;
    red[k].nent = (int)op.nent;
    red[k].gx = op.plane ? op.grid_adj : op.sched.gx[0];
    red[k].plane = op.plane;
    red[k].layout = op.layout;
    red[k].chunk0 = chunks;
    red[k].ec = red_entries_per_cta(red[k].gx);
    chunks += (int)((op.nent + red[k].ec - 1) / red[k].ec);
  }
  P->red_chunks = chunks;
}

// Partial-sum regions and the workspace past the C arena: they depend on
// every op's kernel family and adjoint schedule, so fock_plan_tune redoes them.
static void layout_partials(fock_plan* P) {
  int64_t sum = 0, mx = 0;
  for (PlanOp& op : P->ops) {
    const int64_t part_k = op.plane ? (int64_t)op.grid_adj * op.pg_adj.nent : op.sched.part_entries;
    op.cpart_off = sum;
    sum += part_k;
    mx = std::max(mx, part_k);
  }
  // every op's partials kept until one reduction after the sweep when that
  // costs at most 512 MiB (about 280 MB for the 6-mode cutoff-12 CV-QNN)
  P->reduce_at_end = (double)sum * P->batch * sizeof(double2) <= 512.0 * (1 << 20);
  P->cpart_entries = P->reduce_at_end ? sum : mx;
  size_t o = align256(P->o_cpart + sizeof(double2) * std::max<int64_t>(P->cpart_entries, 1) * P->batch);
  if (P->persist) {
    P->o_sync = o; o = align256(o + (4 + P->ops.size()) * sizeof(unsigned));
    P->o_ppart = o; o = align256(o + sizeof(double2) * std::max<int64_t>(P->ppart_entries, 1));
  }
  P->ws_bytes = o;
  if (P->host) write_red_table(P);
}

// Group consecutive ops into fused tile groups of the forward sweep.  Greedy
// over a valid order:
// take the first op not yet placed; among the three-mode sets that contain its
// modes, pick the one that absorbs the most ready ops (ops whose modes lie in
// the set and whose predecessors -- earlier ops sharing a mode -- are placed
// or absorbed), in program order; a set that absorbs one op leaves it a plain
// op.  The ops are reordered group by group (ops on disjoint modes commute).
static void form_tile_groups(fock_plan* P) {
  const int N = P->N, D = P->D, n = (int)P->ops.size();
  P->groups.clear();
  if (!P->pure || P->dtype != FOCK_C64 || D > 16 || N < 4 || n < 2) return;
  double lg = N * log2((double)D);
  if (lg >= 31.0) return;  // tile offsets are 32-bit
  int64_t ncols = 1;
  for (int k = 0; k < N - 3; ++k) ncols *= D;
  // columns per chunk: 4, or fewer where two CTAs per SM would not fit
  int tc = 4;
  while (tc > 1 && tile_smem_bytes(D, tc) > 113 * 1024) tc /= 2;
  const int64_t nchunks = (ncols + tc - 1) / tc;
  if (nchunks * P->batch < 2 * fock_num_sms()) return;
  for (const PlanOp& op : P->ops)
    if (op.conj || op.owner >= 0) return;
  // predecessors
  std::vector<std::vector<int>> pred(n);
  std::vector<int> last(N, -1);
  for (int i = 0; i < n; ++i) {
    const PlanOp& op = P->ops[i];
    int ms[2] = {op.mode1, op.mode2};
    for (int q = 0; q < 2; ++q)
      if (ms[q] >= 0 && last[ms[q]] >= 0) pred[i].push_back(last[ms[q]]);
    for (int q = 0; q < 2; ++q)
      if (ms[q] >= 0) last[ms[q]] = i;
  }
  std::vector<char> placed(n, 0);
  std::vector<int> order;
  std::vector<fock_plan::Group> groups;
  int first = 0;
  while ((int)order.size() < n) {
    while (placed[first]) ++first;
    const PlanOp& f = P->ops[first];
    std::vector<std::array<int, 3>> cands;
    for (int a = 0; a < N; ++a)
      for (int b = a + 1; b < N; ++b)
        for (int c = b + 1; c < N; ++c) {
          const bool has1 = f.mode1 == a || f.mode1 == b || f.mode1 == c;
          const bool has2 = f.mode2 < 0 || f.mode2 == a || f.mode2 == b || f.mode2 == c;
          if (has1 && has2) cands.push_back({a, b, c});
        }
    std::vector<int> best;
    std::array<int, 3> best_m = cands[0];
    for (const auto& m : cands) {
      std::vector<int> grp;
      std::vector<char> in(n, 0);
      for (int i = first; i < n && (int)grp.size() < TL_MAX_OPS; ++i) {
        if (placed[i]) continue;
        const PlanOp& op = P->ops[i];
        auto inset = [&](int md) { return md < 0 || md == m[0] || md == m[1] || md == m[2]; };
        if (!inset(op.mode1) || !inset(op.mode2)) continue;
        bool ready = true;
        for (int pq : pred[i])
          if (!placed[pq] && !in[pq]) { ready = false; break; }
        if (!ready) continue;
        in[i] = 1;
        grp.push_back(i);
      }
      if (grp.size() > best.size()) { best = grp; best_m = m; }
    }
    if (best.size() >= 2) {
      fock_plan::Group g;
      g.k0 = (int)order.size();
      g.k1 = g.k0 + (int)best.size();
      g.m[0] = best_m[0]; g.m[1] = best_m[1]; g.m[2] = best_m[2];
      groups.push_back(g);
      for (int i : best) { placed[i] = 1; order.push_back(i); }
    } else {
      placed[first] = 1;
      order.push_back(first);
    }
  }
  if (groups.empty()) return;
  std::vector<PlanOp> ops;
  for (int i : order) ops.push_back(P->ops[i]);
  for (size_t gi = 0; gi < groups.size(); ++gi)
    for (int k = groups[gi].k0; k < groups[gi].k1; ++k) ops[k].group = (int)gi;
  P->ops = ops;
  P->groups = groups;
  P->tile_tc = tc;
  // forward CTAs: every chunk in one wave when the resident CTAs allow it
  // (shared memory bounds the CTAs per SM; registers allow 4)
  const int per_sm = std::max(1, std::min(4, (int)((227 * 1024) / tile_smem_bytes(D, tc))));
  P->tile_grid = (int)std::min<int64_t>(nchunks, (int64_t)per_sm * fock_num_sms());
}

extern "C" int fock_plan_create(int num_modes, int cutoff, int pure, int dtype, const fock_gate* gates,
                                int n_gates, int n_params, fock_plan** out) {
  return fock_plan_create_batch(num_modes, cutoff, pure, dtype, gates, n_gates, n_params, 1, out);
}

extern "C" int fock_plan_create_batch(int num_modes, int cutoff, int pure, int dtype, const fock_gate* gates,
                                      int n_gates, int n_params, int batch, fock_plan** out) {
  if (!out) return fock_set_error(FOCK_ERR_INVALID, "null output pointer");
  if (batch < 1 || batch > 65535) return fock_set_error(FOCK_ERR_INVALID, "batch must be in [1, 65535], got %d", batch);
  *out = nullptr;
  if (dtype != FOCK_C64 && dtype != FOCK_C128) return fock_set_error(FOCK_ERR_INVALID, "bad dtype");
  if (cutoff < 1 || cutoff > FOCK_MAX_CUTOFF) return fock_set_error(FOCK_ERR_INVALID, "bad cutoff %d", cutoff);
  if (num_modes < 1 || num_modes > FOCK_MAX_AXES / 2) return fock_set_error(FOCK_ERR_INVALID, "bad number of modes");
  if (n_gates < 0 || (n_gates > 0 && !gates)) return fock_set_error(FOCK_ERR_INVALID, "bad gate list");
  if (n_params < 0) return fock_set_error(FOCK_ERR_INVALID, "bad parameter count");
  const int naxes = pure ? num_modes : 2 * num_modes;
  if (naxes * log2((double)cutoff) > 60.0) return fock_set_error(FOCK_ERR_INVALID, "state too large");

  fock_plan* P = new fock_plan();
  P->batch = batch;
  P->N = num_modes; P->D = cutoff; P->pure = pure; P->dtype = dtype; P->n_params = n_params;
  P->n_gates = n_gates;
  const int N = num_modes, D = cutoff;

  std::vector<std::vector<Pending>> pend(N);
  std::vector<PendingCK> pck;
  std::vector<int> last_op(N, -1);

  auto fail = [&](int code, const char* msg, int g) {
    delete P;
    return fock_set_error(code, "gate %d: %s", g, msg);
  };

  auto flush_ck = [&](size_t idx) {
    // standalone identity op on the pair carrying the cross-Kerr phase
    PendingCK c = pck[idx];
    PlanOp op;
    op.layout = LAYOUT_SUM;
    op.gate = GATE_IDENTITY;
    op.mode1 = c.a;
    op.mode2 = c.b;
    absorb_pending(op, c.a, pend);
    absorb_pending(op, c.b, pend);
    add_term(op, FN_AB, 0, c.pidx);
    P->ops.push_back(op);
    last_op[c.a] = last_op[c.b] = (int)P->ops.size() - 1;
  };

  for (int g = 0; g < n_gates; ++g) {
    const fock_gate& G = gates[g];
    const int two = is_two(G.kind);
    if (G.mode1 < 0 || G.mode1 >= N) return fail(FOCK_ERR_INVALID, "invalid mode", g);
    if (two && (G.mode2 < 0 || G.mode2 >= N || G.mode2 == G.mode1)) return fail(FOCK_ERR_INVALID, "invalid second mode", g);
    const int np = (G.kind == FOCK_ROTATION || G.kind == FOCK_KERR || G.kind == FOCK_CROSS_KERR || G.kind == FOCK_LOSS) ? 1 : 2;
    if (G.pidx < 0 || G.pidx + np > n_params) return fail(FOCK_ERR_INVALID, "parameter index out of range", g);
    if (G.kind == FOCK_LOSS && pure) return fail(FOCK_ERR_UNSUPPORTED, "loss channel in a pure-state circuit", g);
    if (is_diag1(G.kind)) {
      pend[G.mode1].push_back(Pending{G.kind == FOCK_ROTATION ? FN_A : FN_A2, G.pidx});
      continue;
    }
    if (G.kind == FOCK_CROSS_KERR) {
      pck.push_back(PendingCK{G.mode1, G.mode2, G.pidx});
      continue;
    }
    const int layout = gate_layout(G.kind);
    if (!layout) return fail(FOCK_ERR_INVALID, "unknown gate kind", g);
    // cross-Kerr pending on a mode this gate touches must be applied first,
    // unless this gate acts on exactly that pair (then it becomes a phase term)
    PlanOp op;
    op.layout = layout;
    op.gate = G.kind;
    op.mode1 = G.mode1;
    op.mode2 = two ? G.mode2 : -1;
    op.pidx = G.pidx;
    op.n_fused = 1;
    std::vector<PendingCK> keep;
    std::vector<PendingCK> fuse_here;
    for (size_t i = 0; i < pck.size(); ++i) {
      const PendingCK& c = pck[i];
      const bool touches = c.a == G.mode1 || c.b == G.mode1 || (two && (c.a == G.mode2 || c.b == G.mode2));
      if (!touches) { keep.push_back(c); continue; }
      const bool same_pair = two && ((c.a == G.mode1 && c.b == G.mode2) || (c.a == G.mode2 && c.b == G.mode1));
      if (same_pair) fuse_here.push_back(c);
      else {
        pck[i] = c;
        flush_ck(i);
      }
    }
    pck = keep;
    absorb_pending(op, G.mode1, pend);
    if (two) absorb_pending(op, G.mode2, pend);
    for (const PendingCK& c : fuse_here) add_term(op, FN_AB, 0, c.pidx);
    switch (G.kind) {
      case FOCK_DISPLACEMENT:
        add_contrib(op, GC_DM, 0, G.pidx, 1.0);
        add_contrib(op, GC_W_DIFF, FN_A, G.pidx + 1, 1.0);
        break;
      case FOCK_SQUEEZE:
        add_contrib(op, GC_DM, 0, G.pidx, 1.0);
        add_contrib(op, GC_W_DIFF, FN_A, G.pidx + 1, 0.5);
        break;
      case FOCK_BEAMSPLITTER:
        add_contrib(op, GC_DM, 0, G.pidx, 1.0);
        add_contrib(op, GC_W_DIFF, FN_B, G.pidx + 1, 1.0);
        break;
      case FOCK_TWO_MODE_SQUEEZE:
        add_contrib(op, GC_DM, 0, G.pidx, 1.0);
        add_contrib(op, GC_W_DIFF, FN_A, G.pidx + 1, 1.0);
        break;
      case FOCK_MZGATE:
        // MZ(phi_in, phi_ex): R(phi_ex) on mode1 first, carried as a phase term
        add_contrib(op, GC_DM, 0, G.pidx, 1.0);
        add_term(op, FN_A, 0, G.pidx + 1);
        op.n_fused--;  // part of the gate itself
        break;
      case FOCK_LOSS:
        // superoperator on the mode's (ket, bra) pair; dM = d/dT
        add_contrib(op, GC_DM, 0, G.pidx, 1.0);
        break;
      default:
        break;
    }
    P->ops.push_back(op);
    last_op[G.mode1] = (int)P->ops.size() - 1;
    if (two) last_op[G.mode2] = (int)P->ops.size() - 1;
  }
  // leftovers: cross-Kerr as identity ops, then single-mode phases as output
  // terms of the last op on the mode (or an identity op)
  for (size_t i = 0; i < pck.size(); ++i) flush_ck(i);
  pck.clear();
  for (int m = 0; m < N; ++m) {
    if (pend[m].empty()) continue;
    if (last_op[m] < 0) {
      PlanOp op;
      op.layout = LAYOUT_DENSE;
      op.gate = GATE_IDENTITY;
      op.mode1 = m;
      absorb_pending(op, m, pend);
      P->ops.push_back(op);
      last_op[m] = (int)P->ops.size() - 1;
      continue;
    }
    PlanOp& op = P->ops[last_op[m]];
    const int slot_b = (op.layout != LAYOUT_DENSE && op.mode2 == m);
    for (const Pending& p : pend[m]) {
      if (op.gate == FOCK_LOSS) {
        add_loss_terms(op, p.fn, 1, p.pidx);
        continue;
      }
      int fn = p.fn;
      if (slot_b) fn = (fn == FN_A) ? FN_B : FN_B2;
      add_term(op, fn, 1, p.pidx);
    }
    pend[m].clear();
  }

  // state axes of every op; a density matrix applies each unitary op on the
  // ket axes with M and on the bra axes with conj(M) (one matrix, two
  // launches), the loss superoperator once on the mode's (ket, bra) pair
  if (pure) {
    for (PlanOp& op : P->ops) {
      op.axis_a = op.mode1;
      op.axis_b = op.mode2;
    }
  } else {
    std::vector<PlanOp> ex;
    for (const PlanOp& op : P->ops) {
      if (op.gate == FOCK_LOSS) {
        PlanOp l = op;
        l.axis_a = 2 * op.mode1;
        l.axis_b = 2 * op.mode1 + 1;
        ex.push_back(l);
        continue;
      }
      PlanOp ket = op;
      ket.axis_a = 2 * op.mode1;
      ket.axis_b = op.mode2 >= 0 ? 2 * op.mode2 : -1;
      ex.push_back(ket);
      PlanOp bra = op;
      bra.axis_a = 2 * op.mode1 + 1;
      bra.axis_b = op.mode2 >= 0 ? 2 * op.mode2 + 1 : -1;
      bra.conj = 1;
      bra.owner = (int)ex.size() - 1;
      bra.n_fused = 0;
      bra.terms.clear();  // built once, by the ket op
      ex.push_back(bra);
    }
    P->ops = ex;
  }

  // fused three-mode tile groups of the forward sweep (pure complex64 states,
  // cutoff <= 16, enough columns to fill the GPU), with
  // FOCK_GB300_TILE_GROUPS=1 at plan creation; off by default: on the 6-mode
  // cutoff-12 CV-QNN the grouped forward sweep measured 3.5 ms (58 launches)
  // against 2.08 ms for the per-op launches
  const char* tg = getenv("FOCK_GB300_TILE_GROUPS");
  if (tg && strcmp(tg, "1") == 0) form_tile_groups(P);

  // layout of arena / C arena / partials, and tables
  int64_t elems = 1;
  for (int k = 0; k < naxes; ++k) elems *= D;
  P->state_elems = elems;
  // kernel family per op: plane-tile kernels where plane_preferred says so;
  // FOCK_GB300_KERNELS=block / plane forces one family (where it applies)
  const char* kern = getenv("FOCK_GB300_KERNELS");
  const bool use_plane = !(kern && strcmp(kern, "block") == 0);
  const bool force_plane = kern && strcmp(kern, "plane") == 0;
  // persistent sweeps for single circuits whose state is at most
  // FOCK_GB300_SWEEP_MAX_BYTES (default 0: off -- on the 6-mode cutoff-12
  // CV-QNN the per-op launches with programmatic dependent launch measured
  // 2.3 ms per forward against 3.6 ms for the persistent sweep, whose grid
  // barrier alone costs about 3 us per op)
  // FOCK_GB300_MAT32=0 keeps the FP64 matrices in the sweep kernels' staging
  const char* m32 = getenv("FOCK_GB300_MAT32");
  P->mat32 = dtype == FOCK_C64 && !(m32 && atoi(m32) == 0);
  const char* sw = getenv("FOCK_GB300_SWEEP_MAX_BYTES");
  const int64_t sweep_max = sw ? (int64_t)atoll(sw) : 0;
  const int64_t sbytes = elems * (dtype == FOCK_C64 ? 8 : 16);
  // FOCK_GB300_SWEEP_SPIN_LIMIT: polls before a grid barrier of the
  // persistent sweeps gives up (default 2^24; a small value makes a barrier
  // run out, which the error path's tests use)
  const char* sl = getenv("FOCK_GB300_SWEEP_SPIN_LIMIT");
  if (sl) P->spin_limit = (unsigned)strtoul(sl, nullptr, 10);
  if (batch == 1 && sbytes <= sweep_max && dmax_bucket(D) > 0 && P->groups.empty()) {
    P->g_fwd = sweep_grid(dtype, D, 0);
    P->g_bwd = sweep_grid(dtype, D, 1);
    P->persist = P->g_fwd > 0 && P->g_bwd > 0;
  }
  int64_t ppart = 0;
  int64_t arena = 0, carena = 0;
  int n_terms = 0, n_contrib = 0;
  for (size_t k = 0; k < P->ops.size(); ++k) {
    PlanOp& op = P->ops[k];
    op.nent = layout_entries(op.layout, D);
    if (op.owner >= 0) {
      const PlanOp& ow = P->ops[op.owner];
      op.m_off = ow.m_off;
      op.dm_off = ow.dm_off;
      op.scratch_off = ow.scratch_off;
    } else {
      op.m_off = arena;
      arena += op.nent;
      const bool has_dm = op.gate != GATE_IDENTITY;
      if (has_dm) { op.dm_off = arena; arena += op.nent; }
      const int64_t ns = build_scratch_entries(op.gate, D);
      if (ns > 0) { op.scratch_off = arena; arena += ns; }
    }
    if (op.layout == LAYOUT_DENSE) op.view = make_view1(naxes, D, op.axis_a);
    else {
      int a = op.axis_a, b = op.axis_b;
      op.swap = a > b;
      op.view = make_view2(naxes, D, std::min(a, b), std::max(a, b));
    }
    op.sched = make_adj_sched(dtype, op.view, D, op.layout, batch, op.adj_ctas);
    op.plane_ok = use_plane && make_plane_geom(dtype, op.view, D, op.layout, op.swap, 0, &op.pg_fwd) &&
                  make_plane_geom(dtype, op.view, D, op.layout, op.swap, 1, &op.pg_adj);
    if (op.plane_ok) {
      op.grid_fwd = plane_grid(dtype, op.pg_fwd, 0, batch);
      op.grid_adj = plane_grid(dtype, op.pg_adj, 1, batch);
    }
    op.plane = op.plane_ok && (force_plane || plane_preferred(op.layout, op.view));
    if (P->persist) {
      op.psched = make_adj_sched_grid(dtype, op.view, D, op.layout, P->g_bwd);
      op.ppart_off = ppart;
      ppart += op.psched.part_entries;
    }
    op.c_off = carena;
    carena += op.nent;
    n_terms += (int)op.terms.size();
    n_contrib += (int)op.contribs.size();
    // flops: 8 real flops per complex multiply-add
    int64_t macs_per_col = op.layout == LAYOUT_DENSE ? (int64_t)D * D : blk_total(D);
    P->flops_fwd += 8 * macs_per_col * op.view.ncols;
  }
  P->arena_entries = arena;
  P->carena_entries = carena;
  P->n_terms = n_terms;
  P->n_contrib = n_contrib;
  const int n_ops = (int)P->ops.size();
  size_t o = 0;
  P->n_jobs = 0;
  for (const PlanOp& op : P->ops) P->n_jobs += op.owner < 0;
  P->o_jobs = o; o = align256(o + sizeof(BuildJob) * std::max(P->n_jobs, 1));
  P->o_terms = o; o = align256(o + sizeof(PhaseTerm) * std::max(n_terms, 1));
  P->o_gops = o; o = align256(o + sizeof(GradOp) * std::max(n_ops, 1));
  P->o_contrib = o; o = align256(o + sizeof(GradContrib) * std::max(n_contrib, 1));
  P->o_pstart = o; o = align256(o + sizeof(int) * (n_params + 1));
  P->o_plist = o; o = align256(o + sizeof(int) * std::max(n_contrib, 1));
  if (P->persist) { P->o_sweep = o; o = align256(o + sizeof(SweepOp) * std::max(n_ops, 1)); }
  P->o_red = o; o = align256(o + sizeof(RedOp) * std::max(n_ops, 1));
  P->tables_bytes = o;
  P->o_arena = o; o = align256(o + sizeof(double2) * arena * batch);
  P->o_carena = o; o = align256(o + sizeof(double2) * std::max<int64_t>(carena, 1) * batch);
  if (P->mat32) { P->o_arena32 = o; o = align256(o + sizeof(float2) * std::max<int64_t>(arena, 1) * batch); }
  P->o_cpart = o;
  P->ppart_entries = ppart;
  layout_partials(P);

  if (cudaHostAlloc((void**)&P->host, P->tables_bytes, cudaHostAllocDefault) != cudaSuccess) {
    // fall back to pageable memory (copies are then synchronous)
    cudaGetLastError();
    P->host = (unsigned char*)malloc(P->tables_bytes);
    if (!P->host) { delete P; return fock_set_error(FOCK_ERR_INVALID, "out of host memory"); }
  }
  memset(P->host, 0, P->tables_bytes);
  BuildJob* jobs = (BuildJob*)(P->host + P->o_jobs);
  PhaseTerm* terms = (PhaseTerm*)(P->host + P->o_terms);
  GradOp* gops = (GradOp*)(P->host + P->o_gops);
  GradContrib* contrib = (GradContrib*)(P->host + P->o_contrib);
  int* pstart = (int*)(P->host + P->o_pstart);
  int* plist = (int*)(P->host + P->o_plist);
  int t = 0, c = 0, nj = 0;
  std::vector<std::vector<int>> by_param(n_params);
  for (int k = 0; k < n_ops; ++k) {
    PlanOp& op = P->ops[k];
    if (op.owner < 0) {  // builds its matrix (bra-side ops reuse the ket op's)
      BuildJob& J = jobs[nj++];
      J.gate = op.gate;
      J.layout = op.layout;
      J.D = D;
      J.pidx = op.pidx;
      J.v0 = J.v1 = 0.0;
      J.term0 = t;
      J.nterm = (int)op.terms.size();
      J.m_off = op.m_off;
      J.dm_off = op.dm_off;
      J.scratch_off = op.scratch_off;
      for (const PhaseTerm& pt : op.terms) terms[t++] = pt;
    }
    GradOp& go = gops[k];
    go.layout = op.layout;
    go.D = D;
    go.m_off = op.m_off;
    go.dm_off = op.dm_off;
    go.c_off = op.c_off;
    go.nent = (int)op.nent;
    go.conj = op.conj;
    for (GradContrib gc : op.contribs) {
      gc.op = k;
      contrib[c] = gc;
      by_param[gc.pidx].push_back(c);
      ++c;
    }
  }
  // longest builds first (one CTA per job): the CTA scheduler gives the
  // first CTAs an SM each, so the jobs that share an SM are the short ones
  auto build_cost = [](const BuildJob& J) {
    switch (J.gate) {
      case FOCK_MZGATE: return 4;
      case FOCK_BEAMSPLITTER:
      case FOCK_TWO_MODE_SQUEEZE: return 3;
      case FOCK_LOSS: return 2;
      default: return J.layout == LAYOUT_DENSE ? 0 : 1;
    }
  };
  std::stable_sort(jobs, jobs + nj,
                   [&](const BuildJob& a, const BuildJob& b) { return build_cost(a) > build_cost(b); });
  write_red_table(P);
  if (P->persist) {
    SweepOp* sw_ops = (SweepOp*)(P->host + P->o_sweep);
    for (int k = 0; k < n_ops; ++k) {
      const PlanOp& op = P->ops[k];
      SweepOp& s = sw_ops[k];
      s.view = op.view;
      s.layout = op.layout;
      s.mflags = op_flags(op);
      s.m_off = op.m_off;
      s.c_off = op.c_off;
      s.part_base = op.ppart_off;
      s.nent = (int)op.nent;
      s.fwd_nx = (int)((op.view.ncols + 255) / 256);
      s.sc = op.psched;
    }
  }
  int q = 0;
  for (int p = 0; p < n_params; ++p) {
    pstart[p] = q;
    for (int ci : by_param[p]) plist[q++] = ci;
  }
  pstart[n_params] = q;
  *out = P;
  return FOCK_OK;
}

extern "C" void fock_plan_destroy(fock_plan* P) {
  if (!P) return;
  for (cudaEvent_t e : P->ev_fwd) cudaEventDestroy(e);
  for (cudaEvent_t e : P->ev_bwd) cudaEventDestroy(e);
  if (P->host) {
    if (cudaFreeHost(P->host) != cudaSuccess) {
      cudaGetLastError();
      free(P->host);
    }
  }
  delete P;
}

extern "C" int fock_plan_get_info(const fock_plan* P, fock_plan_info* info) {
  if (!P || !info) return fock_set_error(FOCK_ERR_INVALID, "null argument");
  info->n_ops = (int32_t)P->ops.size();
  info->n_gates = P->n_gates;
  info->state_elems = P->state_elems;
  info->state_bytes = P->state_elems * (P->dtype == FOCK_C64 ? 8 : 16);
  info->workspace_bytes = (int64_t)P->ws_bytes;
  info->flops_fwd = P->flops_fwd * P->batch;
  info->bytes_fwd = 2 * info->state_bytes * (int64_t)P->ops.size() * P->batch;
  info->batch = P->batch;
  return FOCK_OK;
}

extern "C" int fock_plan_op_group(const fock_plan* P, int k, int* group, int* first, int* count) {
  if (!P || k < 0 || k >= (int)P->ops.size()) return fock_set_error(FOCK_ERR_INVALID, "bad op index");
  const int gi = P->ops[k].group;
  if (group) *group = gi;
  if (first) *first = gi >= 0 ? P->groups[gi].k0 : k;
  if (count) *count = gi >= 0 ? P->groups[gi].k1 - P->groups[gi].k0 : 1;
  return FOCK_OK;
}

extern "C" int fock_plan_op(const fock_plan* P, int k, int* kind, int* mode1, int* mode2, int* n_fused) {
  if (!P || k < 0 || k >= (int)P->ops.size()) return fock_set_error(FOCK_ERR_INVALID, "bad op index");
  const PlanOp& op = P->ops[k];
  if (kind) *kind = op.layout;
  if (mode1) *mode1 = op.mode1;
  if (mode2) *mode2 = op.mode2;
  if (n_fused) *n_fused = op.n_fused;
  return FOCK_OK;
}

// ---------------------------------------------------------------------------
// execution
// ---------------------------------------------------------------------------
// complex64 copies of the built matrices (every arena entry of every circuit)
__global__ void arena32_kernel(const double2* __restrict__ a, float2* __restrict__ o, int64_t n) {
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += step)
    o[i] = make_float2((float)a[i].x, (float)a[i].y);
}

static int upload_and_build(fock_plan* P, const double* params, unsigned char* ws, int with_deriv,
                            cudaStream_t st) {
  FOCK_CUDA_TRY(cudaMemcpyAsync(ws, P->host, P->tables_bytes, cudaMemcpyHostToDevice, st));
  const int n_ops = (int)P->ops.size();
  if (!with_deriv) {
    // forward only needs M: a job table with dm_off = -1 would need a second
    // table; building dM as well costs one extra matrix write per op and keeps
    // one table
  }
  int rc = launch_build_jobs((const BuildJob*)(ws + P->o_jobs), P->n_jobs, (const PhaseTerm*)(ws + P->o_terms),
                             params, (double2*)(ws + P->o_arena), st, P->batch, P->n_params, P->arena_entries);
  if (rc || !P->mat32) return rc;
  const int64_t n = P->arena_entries * P->batch;
  const int64_t blocks = std::min<int64_t>((n + 255) / 256, 4096);
  arena32_kernel<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, st>>>((const double2*)(ws + P->o_arena),
                                                                        (float2*)(ws + P->o_arena32), n);
  FOCK_LAUNCH_CHECK("arena32_kernel");
  return FOCK_OK;
}

// grid-barrier words of a persistent sweep, cleared before every launch
static int sweep_sync(fock_plan* P, unsigned char* ws, cudaStream_t st, SweepSync* s) {
  unsigned* w = (unsigned*)(ws + P->o_sync);
  FOCK_CUDA_TRY(cudaMemsetAsync(w, 0, (4 + P->ops.size()) * sizeof(unsigned), st));
  s->count = w;
  s->gen = w + 1;
  s->err = (int*)(w + 2);
  s->items = w + 4;
  s->spin_limit = P->spin_limit;
  return FOCK_OK;
}

struct SweepCtx {
  fock_plan* P;
  const double2* arena;
  const float2* arena32;  // complex64 copies (mat32 plans), or null
  BatchArg bt;
  int64_t sb;  // bytes of one slot (whole batch)
  cudaStream_t st;
};

static int sweep_ctx(fock_plan* P, unsigned char* ws, cudaStream_t st, SweepCtx* c) {
  const int esz = P->dtype == FOCK_C64 ? 8 : 16;
  c->P = P;
  c->sb = P->state_elems * esz * P->batch;
  c->arena = (const double2*)(ws + P->o_arena);
  c->arena32 = P->mat32 ? (const float2*)(ws + P->o_arena32) : nullptr;
  c->bt.nb = P->batch;
  c->bt.state_stride = P->state_elems;
  c->bt.mat_stride = P->arena_entries;
  c->bt.part_stride = P->cpart_entries;
  c->st = st;
  return FOCK_OK;
}

// kernel arguments of ops [k0, k1) of tile group gi (stores left unset: -1)
static void tile_arg(const fock_plan* P, int gi, int k0, int k1, TileGroupArg* a) {
  memset(a, 0, sizeof(*a));
  const fock_plan::Group& G = P->groups[gi];
  const int N = P->N, D = P->D;
  auto stride = [&](int m) {
    int64_t s = 1;
    for (int q = m + 1; q < N; ++q) s *= D;
    return s;
  };
  a->D = D;
  a->T = D * D * D;
  a->nops = k1 - k0;
  a->TC = P->tile_tc;
  a->lgTC = 0;
  while ((1 << a->lgTC) < a->TC) ++a->lgTC;
  for (int i = 0; i < 3; ++i) a->S[i] = stride(G.m[i]);
  int nr = 0;
  for (int m = 0; m < N; ++m)
    if (m != G.m[0] && m != G.m[1] && m != G.m[2]) a->rest_stride[nr++] = stride(m);
  a->nrest = nr;
  a->c_fast = G.m[2] != N - 1;
  a->ncols = 1;
  for (int q = 0; q < N - 3; ++q) a->ncols *= D;
  a->nchunks = (a->ncols + a->TC - 1) / a->TC;
  a->slot_elems = P->state_elems * P->batch;
  auto ax = [&](int m) { return m == G.m[0] ? 0 : (m == G.m[1] ? 1 : 2); };
  for (int k = k0; k < k1; ++k) {
    const PlanOp& op = P->ops[k];
    TileOp& t = a->ops[k - k0];
    t.layout = op.layout;
    if (op.layout == LAYOUT_DENSE) {
      t.ta = ax(op.mode1);
      t.tb = -1;
      t.swap = 0;
    } else {
      const int x1 = ax(op.mode1), x2 = ax(op.mode2);
      t.ta = std::min(x1, x2);
      t.tb = std::max(x1, x2);
      t.swap = x1 > x2;
    }
    t.m_off = op.m_off;
    t.store_slot = -1;
  }
}

// the matrix of op k for the sweep kernels, and its staging flags
static const double2* sweep_mat(const SweepCtx& c, const PlanOp& op) {
  if (c.arena32) return reinterpret_cast<const double2*>(c.arena32 + op.m_off);
  return c.arena + op.m_off;
}
static int sweep_flags(const SweepCtx& c, const PlanOp& op) { return op_flags(op) | (c.arena32 ? MF_F32 : 0); }

static int apply_op(const SweepCtx& c, int k, const void* in, void* out) {
  const PlanOp& op = c.P->ops[k];
  if (op.plane)
    return launch_plane_apply(c.P->dtype, in, out, op.pg_fwd, op.grid_fwd, sweep_mat(c, op), sweep_flags(c, op),
                              c.st, c.bt);
  return launch_apply(c.P->dtype, in, out, op.view, c.P->D, op.layout, sweep_mat(c, op), sweep_flags(c, op),
                      c.st, c.bt);
}

extern "C" int fock_plan_forward(fock_plan* P, const double* params, const void* state_in, void* states,
                                 int store_every, void* workspace, void* stream) {
  if (!P) return fock_set_error(FOCK_ERR_INVALID, "null plan");
  if (!state_in || !states || !workspace) return fock_set_error(FOCK_ERR_INVALID, "null buffer");
  if (P->n_params > 0 && !params) return fock_set_error(FOCK_ERR_INVALID, "null parameter array");
  if (store_every < 0) return fock_set_error(FOCK_ERR_INVALID, "store_every must be >= 0");
  cudaStream_t st = (cudaStream_t)stream;
  unsigned char* ws = (unsigned char*)workspace;
  int rc = upload_and_build(P, params, ws, 0, st);
  if (rc) return rc;
  SweepCtx c;
  sweep_ctx(P, ws, st, &c);
  const void* cur = state_in;
  const int n_ops = (int)P->ops.size();
  if (P->persist && !P->timing && store_every <= 1 && n_ops > 0) {
    SweepSync sync;
    if ((rc = sweep_sync(P, ws, st, &sync))) return rc;
    const int esz = P->dtype == FOCK_C64 ? 8 : 16;
    return launch_sweep_forward(P->dtype, P->D, (const SweepOp*)(ws + P->o_sweep), n_ops, store_every, state_in,
                                states, c.sb / esz, c.arena, sync, P->g_fwd, st);
  }
  if (P->timing) {
    if ((rc = ensure_events(P->ev_fwd, n_ops + 1))) return rc;
    P->fwd_recorded = 0;
  }
  for (int k = 0; k < n_ops; ++k) {
    const PlanOp& op = P->ops[k];
    if (op.group >= 0 && !P->timing && P->groups[op.group].k0 == k) {
      // a whole tile group in one launch; it writes the outputs the sweep
      // keeps: every op's (store_every 1), the checkpoints, and the last op's
      const int k1 = P->groups[op.group].k1;
      TileGroupArg a;
      tile_arg(P, op.group, k, k1, &a);
      for (int j = k; j < k1; ++j) {
        const bool keep = store_every == 1 || j == k1 - 1 ||
                          (store_every > 1 && ((j + 1) % store_every == 0 || j == n_ops - 1));
        a.ops[j - k].store_slot = keep ? out_slot(j, n_ops, store_every) : -1;
      }
      c.bt.pdl = k > 0;
      if ((rc = launch_tile_forward(a, cur, states, c.arena, P->tile_grid, st, c.bt))) return rc;
      cur = (char*)states + out_slot(k1 - 1, n_ops, store_every) * c.sb;
      k = k1 - 1;
      continue;
    }
    void* dst = (char*)states + out_slot(k, n_ops, store_every) * c.sb;
    if (P->timing && (rc = record_event(P->ev_fwd[k], st))) return rc;
    // the first op follows the matrix build in plain stream order; later ops
    // overlap their launch with the previous op's tail (not across the
    // timing events)
    c.bt.pdl = k > 0 && !P->timing;
    if ((rc = apply_op(c, k, cur, dst))) return rc;
    cur = dst;
  }
  if (P->timing) {
    if ((rc = record_event(P->ev_fwd[n_ops], st))) return rc;
    P->fwd_recorded = 1;
  }
  return FOCK_OK;
}

static int param_grads(fock_plan* P, unsigned char* ws, const SweepCtx& c, double* grad_params, cudaStream_t st) {
  if (P->n_params > 0)
    return launch_param_grads((const GradOp*)(ws + P->o_gops), (const GradContrib*)(ws + P->o_contrib),
                              (const int*)(ws + P->o_pstart), (const int*)(ws + P->o_plist), P->n_params,
                              (const PhaseTerm*)(ws + P->o_terms), c.arena, (const double2*)(ws + P->o_carena),
                              grad_params, st, P->batch, P->arena_entries, P->carena_entries);
  return FOCK_OK;
}

// one adjoint sweep in progress: lam holds dL/d(output of the next op to
// process), other receives dL/d(its input)
struct BwdCtx {
  fock_plan* P;
  SweepCtx c;
  unsigned char* ws;
  double2* cpart;
  void* lam;
  void* other;
  int pdl;
};

static int adjoint_op(BwdCtx& b, int k, const void* psi_in) {
  fock_plan* P = b.P;
  const PlanOp& op = P->ops[k];
  cudaStream_t st = b.c.st;
  int rc;
  if (P->timing && (rc = record_event(P->ev_bwd[k + 1], st))) return rc;
  double2* cout = (double2*)(b.ws + P->o_carena) + op.c_off;
  double2* part = b.cpart + (P->reduce_at_end ? op.cpart_off : 0);
  if (op.plane) {
    rc = launch_plane_adjoint(P->dtype, psi_in, b.lam, b.other, op.pg_adj, op.grid_adj, sweep_mat(b.c, op),
                              sweep_flags(b.c, op), part, st, b.c.bt);
    if (rc) return rc;
    if (!P->reduce_at_end)
      rc = launch_reduce_partials(part, op.grid_adj, op.nent, cout, st, P->batch, P->cpart_entries,
                                  P->carena_entries, b.pdl);
  } else {
    rc = launch_adjoint_partials(P->dtype, psi_in, b.lam, b.other, op.view, P->D, op.layout, sweep_mat(b.c, op),
                                 sweep_flags(b.c, op), part, op.sched, st, b.c.bt);
    if (rc) return rc;
    if (!P->reduce_at_end)
      rc = launch_reduce_sched(part, op.sched, P->D, op.layout, cout, st, P->batch, P->cpart_entries,
                               P->carena_entries, b.pdl);
  }
  if (rc) return rc;
  b.c.bt.pdl = b.pdl;
  std::swap(b.lam, b.other);
  return FOCK_OK;
}

static int forward_op(BwdCtx& b, int j, const void* in, void* out) {
  const int rc = apply_op(b.c, j, in, out);
  b.c.bt.pdl = b.pdl;
  return rc;
}

// Adjoint of ops [s0, e) whose first input is x, recomputing the states in
// between into slots taken from `pool` (returned afterwards).
//  - n - 1 <= F free slots: recompute the n - 1 inner states once, keep them.
//  - otherwise split at m boundaries (recomputed through two scratch slots);
//    chunk i is processed while boundaries 1..i are held, so it may keep up
//    to F - i states: the last chunks take F - i + 1 ops, the first chunk the
//    rest.  The fewest boundaries that cover the segment this way are used
//    (one recomputation of the segment plus one of each chunk).
//  - if no split covers it, one boundary F ops before the end: that chunk is
//    processed directly, the front part again by this rule.
static int bwd_range(BwdCtx& b, int s0, int e, const void* x, std::vector<void*>& pool) {
  const int n = e - s0;
  if (n <= 0) return FOCK_OK;
  const int F = (int)pool.size();
  int rc;
  if (n - 1 <= F) {
    std::vector<void*> sl(pool.end() - (n - 1), pool.end());
    pool.resize(F - (n - 1));
    const void* cur = x;
    for (int j = s0; j < e - 1; ++j) {
      if ((rc = forward_op(b, j, cur, sl[j - s0]))) return rc;
      cur = sl[j - s0];
    }
    for (int k = e - 1; k >= s0; --k)
      if ((rc = adjoint_op(b, k, k == s0 ? x : sl[k - s0 - 1]))) return rc;
    pool.insert(pool.end(), sl.begin(), sl.end());
    return FOCK_OK;
  }
  if (F < 3) return fock_set_error(FOCK_ERR_INVALID, "recomputing a segment of %d ops needs at least 3 slots", n);
  int m = 0;
  for (int t = 1; t <= F - 2 && t <= n - 1 && !m; ++t) {
    int64_t cap = 0;
    for (int i = 0; i <= t; ++i) cap += F - i + 1;
    if (cap >= n) m = t;
  }
  std::vector<int> start;
  if (m) {
    start.assign(m + 2, 0);
    start[0] = s0;
    start[m + 1] = e;
    for (int i = m; i >= 1; --i) start[i] = start[i + 1] - (F - i + 1);
  } else {
    m = 1;
    start = {s0, e - F, e};
  }
  std::vector<void*> bound(m + 1, nullptr);
  for (int i = 1; i <= m; ++i) { bound[i] = pool.back(); pool.pop_back(); }
  void* scratch[2] = {pool[pool.size() - 1], pool[pool.size() - 2]};
  const void* cur = x;
  int nb = 1;  // next boundary to fill
  for (int j = s0; j < start[m]; ++j) {
    void* dst = (j + 1 == start[nb]) ? bound[nb] : scratch[j & 1];
    if ((rc = forward_op(b, j, cur, dst))) return rc;
    if (j + 1 == start[nb]) ++nb;
    cur = dst;
  }
  for (int i = m; i >= 0; --i) {
    if ((rc = bwd_range(b, start[i], start[i + 1], i == 0 ? x : bound[i], pool))) return rc;
    if (i >= 1) pool.push_back(bound[i]);
  }
  return FOCK_OK;
}

extern "C" int fock_plan_backward(fock_plan* P, const double* params, const void* state_in,
                                  const void* states, int store_every, void* seg, void* grad_state,
                                  void* grad_tmp, double* grad_params, void* workspace, void* stream) {
  return fock_plan_backward_recompute(P, params, state_in, states, store_every, seg,
                                      store_every > 1 ? store_every - 1 : 0, grad_state, grad_tmp, grad_params, 0,
                                      workspace, stream);
}

extern "C" int fock_plan_backward_recompute(fock_plan* P, const double* params, const void* state_in,
                                            const void* states, int store_every, void* seg, int seg_slots,
                                            void* grad_state, void* grad_tmp, double* grad_params, int flags,
                                            void* workspace, void* stream) {
  if (!P) return fock_set_error(FOCK_ERR_INVALID, "null plan");
  if (!state_in || !states || !grad_state || !grad_tmp || !workspace)
    return fock_set_error(FOCK_ERR_INVALID, "null buffer");
  if (store_every < 1) return fock_set_error(FOCK_ERR_INVALID, "the adjoint sweep needs store_every >= 1");
  if (store_every > 1 && (!seg || seg_slots < 1))
    return fock_set_error(FOCK_ERR_INVALID, "checkpointed sweep needs a segment buffer");
  if (P->n_params > 0 && (!params || !grad_params)) return fock_set_error(FOCK_ERR_INVALID, "null parameter array");
  cudaStream_t st = (cudaStream_t)stream;
  unsigned char* ws = (unsigned char*)workspace;
  int rc = 0;
  // the forward sweep builds M and dM: reuse them when the caller says the
  // workspace still holds that sweep's build for these parameters
  if (!(flags & FOCK_BACKWARD_REUSE_BUILD) && (rc = upload_and_build(P, params, ws, 1, st))) return rc;
  SweepCtx c;
  sweep_ctx(P, ws, st, &c);
  const int n_ops = (int)P->ops.size();
  const int K = store_every;
  if (P->persist && !P->timing && K == 1 && n_ops > 0) {
    SweepSync sync;
    if ((rc = sweep_sync(P, ws, st, &sync))) return rc;
    const int esz = P->dtype == FOCK_C64 ? 8 : 16;
    rc = launch_sweep_backward(P->dtype, P->D, (const SweepOp*)(ws + P->o_sweep), n_ops, state_in, states,
                               c.sb / esz, grad_state, grad_tmp, c.arena, (double2*)(ws + P->o_ppart),
                               (double2*)(ws + P->o_carena), P->carena_entries, sync, P->g_bwd, st);
    if (rc) return rc;
    // op n-1 reads grad_state, writes grad_tmp; the final lam_in is in
    // grad_state when n_ops is even
    if (n_ops & 1) FOCK_CUDA_TRY(cudaMemcpyAsync(grad_state, grad_tmp, c.sb, cudaMemcpyDeviceToDevice, st));
    return param_grads(P, ws, c, grad_params, st);
  }
  if (P->timing) {
    if ((rc = ensure_events(P->ev_bwd, n_ops + 1))) return rc;
    P->bwd_recorded = 0;
  }
  BwdCtx b;
  b.P = P;
  b.c = c;
  b.ws = ws;
  b.cpart = (double2*)(ws + P->o_cpart);
  b.lam = grad_state;
  b.other = grad_tmp;
  // programmatic dependent launch for every sweep kernel but the first one
  // after the matrix build (and none around timing events)
  b.pdl = !P->timing;
  b.c.bt.pdl = 0;
  if (K == 1) {
    for (int k = n_ops - 1; k >= 0; --k)
      if ((rc = adjoint_op(b, k, k == 0 ? state_in : (const char*)states + (int64_t)(k - 1) * c.sb))) return rc;
  } else {
    std::vector<void*> pool;
    for (int i = seg_slots - 1; i >= 0; --i) pool.push_back((char*)seg + (int64_t)i * c.sb);
    const int nseg = (n_ops + K - 1) / K;
    for (int sgi = nseg - 1; sgi >= 0; --sgi) {
      const int s0 = sgi * K, e = std::min(s0 + K, n_ops);
      const void* seg_in = sgi == 0 ? state_in : (const char*)states + (int64_t)(sgi - 1) * c.sb;
      if ((rc = bwd_range(b, s0, e, seg_in, pool))) return rc;
    }
  }
  void* lam = b.lam;
  if (P->timing) {
    if ((rc = record_event(P->ev_bwd[0], st))) return rc;
    P->bwd_recorded = 1;
  }
  if (P->reduce_at_end && n_ops > 0) {
    rc = launch_reduce_ops((const RedOp*)(ws + P->o_red), n_ops, P->red_chunks, P->D, b.cpart,
                           (double2*)(ws + P->o_carena), st, P->batch, P->cpart_entries, P->carena_entries);
    if (rc) return rc;
  }
  if (lam != grad_state) FOCK_CUDA_TRY(cudaMemcpyAsync(grad_state, lam, c.sb, cudaMemcpyDeviceToDevice, st));
  return param_grads(P, ws, c, grad_params, st);
}

extern "C" int fock_plan_tune(fock_plan* P, int k, int family, int adj_ctas_per_sm, int plane_tile_columns) {
  if (!P || k < 0 || k >= (int)P->ops.size()) return fock_set_error(FOCK_ERR_INVALID, "bad op index");
  PlanOp& op = P->ops[k];
  if (family > 1) return fock_set_error(FOCK_ERR_INVALID, "kernel family must be 0 (block) or 1 (plane)");
  if (family == 1 && !op.plane_ok) return fock_set_error(FOCK_ERR_UNSUPPORTED, "op %d has no plane-tile kernel", k);
  if (adj_ctas_per_sm < 0 || adj_ctas_per_sm > 64)
    return fock_set_error(FOCK_ERR_INVALID, "adjoint CTAs per SM must be in [1, 64]");
  if (plane_tile_columns && (plane_tile_columns < 8 || plane_tile_columns > 32))
    return fock_set_error(FOCK_ERR_INVALID, "plane tile columns must be in [8, 32]");
  if (plane_tile_columns && op.plane_ok && op.layout != LAYOUT_DENSE && plane_tile_columns != (op.pl_tc ? op.pl_tc : 32)) {
    PlaneGeom f, a;
    if (!make_plane_geom(P->dtype, op.view, P->D, op.layout, op.swap, 0, &f, plane_tile_columns) ||
        !make_plane_geom(P->dtype, op.view, P->D, op.layout, op.swap, 1, &a, plane_tile_columns))
      return fock_set_error(FOCK_ERR_UNSUPPORTED, "op %d: no plane geometry with %d tile columns", k,
                            plane_tile_columns);
    op.pg_fwd = f;
    op.pg_adj = a;
    op.grid_fwd = plane_grid(P->dtype, f, 0, P->batch);
    op.grid_adj = plane_grid(P->dtype, a, 1, P->batch);
    op.pl_tc = plane_tile_columns;
  }
  if (family >= 0) op.plane = family;
  if (adj_ctas_per_sm > 0) {
    op.adj_ctas = adj_ctas_per_sm;
    op.sched = make_adj_sched(P->dtype, op.view, P->D, op.layout, P->batch, adj_ctas_per_sm);
  }
  layout_partials(P);
  return FOCK_OK;
}

extern "C" int fock_plan_op_config(const fock_plan* P, int k, int* family, int* adj_ctas_per_sm, int* plane_ok,
                                   int* plane_tile_columns) {
  if (!P || k < 0 || k >= (int)P->ops.size()) return fock_set_error(FOCK_ERR_INVALID, "bad op index");
  const PlanOp& op = P->ops[k];
  if (family) *family = op.plane;
  if (adj_ctas_per_sm) *adj_ctas_per_sm = op.adj_ctas;
  if (plane_ok) *plane_ok = op.plane_ok;
  if (plane_tile_columns) *plane_tile_columns = op.plane_ok ? op.pg_fwd.TC : 0;
  return FOCK_OK;
}

extern "C" int fock_plan_sweep_status(const fock_plan* P, const void* workspace, int* grids, int* error) {
  if (!P) return fock_set_error(FOCK_ERR_INVALID, "null plan");
  if (grids) {
    grids[0] = P->persist ? P->g_fwd : 0;
    grids[1] = P->persist ? P->g_bwd : 0;
  }
  if (error) {
    *error = 0;
    if (P->persist) {
      if (!workspace) return fock_set_error(FOCK_ERR_INVALID, "null workspace");
      FOCK_CUDA_TRY(cudaMemcpy(error, (const unsigned char*)workspace + P->o_sync + 2 * sizeof(unsigned),
                               sizeof(int), cudaMemcpyDeviceToHost));
    }
  }
  return FOCK_OK;
}

extern "C" int fock_plan_enable_timing(fock_plan* P, int enable) {
  if (!P) return fock_set_error(FOCK_ERR_INVALID, "null plan");
  P->timing = enable ? 1 : 0;
  return FOCK_OK;
}

extern "C" int fock_plan_op_times(fock_plan* P, float* fwd_ms, float* bwd_ms) {
  if (!P) return fock_set_error(FOCK_ERR_INVALID, "null plan");
  const int n = (int)P->ops.size();
  if (fwd_ms) {
    if (!P->fwd_recorded) return fock_set_error(FOCK_ERR_INVALID, "no timed forward sweep recorded");
    for (int k = 0; k < n; ++k) FOCK_CUDA_TRY(cudaEventElapsedTime(&fwd_ms[k], P->ev_fwd[k], P->ev_fwd[k + 1]));
  }
  if (bwd_ms) {
    if (!P->bwd_recorded) return fock_set_error(FOCK_ERR_INVALID, "no timed backward sweep recorded");
    // ev_bwd[k+1] was recorded before op k's adjoint, ev_bwd[k] after it
    for (int k = 0; k < n; ++k) FOCK_CUDA_TRY(cudaEventElapsedTime(&bwd_ms[k], P->ev_bwd[k + 1], P->ev_bwd[k]));
  }
  return FOCK_OK;
}
