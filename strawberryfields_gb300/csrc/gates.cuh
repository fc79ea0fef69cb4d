// Gate-matrix build jobs shared by the builder (gates.cu), the circuit plan
// (plan.cu) and the parameter-gradient kernel.
#pragma once
#include "fock_common.cuh"

// storage layout of a built matrix
#define LAYOUT_DENSE 1  // D x D row-major [out][in] on one axis
#define LAYOUT_SUM 2    // photon-number-sum blocks on two axes
#define LAYOUT_DIFF 3   // photon-number-difference blocks on two axes

// phase-term index functions f(coords) of an entry's (axis-1, axis-2) coordinates
#define FN_A 0
#define FN_A2 1
#define FN_B 2
#define FN_B2 3
#define FN_AB 4

__host__ __device__ __forceinline__ double phase_fn(int fn, int a, int b) {
  switch (fn) {
    case FN_A: return (double)a;
    case FN_A2: return (double)a * a;
    case FN_B: return (double)b;
    case FN_B2: return (double)b * b;
    default: return (double)a * b;
  }
}

// exp(i * value * f(coords)) applied to the input (side 0) or output (side 1)
// coordinates of every entry.  value = params[pidx] when pidx >= 0; neg
// negates it (the bra half of a phase on a density-matrix superoperator).
struct PhaseTerm {
  int fn;
  int side;
  int pidx;
  int neg;
  double value;
};

#define GATE_IDENTITY 0  // pure-phase op: U = identity in its layout

struct BuildJob {
  int gate;     // FOCK_* base gate or GATE_IDENTITY
  int layout;   // LAYOUT_*
  int D;
  int pidx;     // p0 = params[pidx], p1 = params[pidx+1]; < 0: use v0, v1
  double v0, v1;
  int term0, nterm;
  int64_t m_off;        // matrix (double2 units) in the arena
  int64_t dm_off;       // derivative wrt p0, or -1
  int64_t scratch_off;  // extended-cutoff scratch, or -1
};

// gradient contribution types (parameter-gradient kernel)
#define GC_DM 0        // Re sum C * dM
#define GC_W_IN 1      // Re sum C * M * i * scale * f(in)
#define GC_W_OUT 2     // Re sum C * M * i * scale * f(out)
#define GC_W_DIFF 3    // Re sum C * M * i * scale * (f(out) - f(in))

struct GradContrib {
  int op;       // op index (matrix + C offsets through ops table)
  int type;
  int fn;
  int pidx;     // destination parameter
  double scale;
};

struct GradOp {
  int layout;
  int D;
  int64_t m_off, dm_off;  // arena offsets
  int64_t c_off;          // offset of the reduced C matrix (double2) in the C arena
  int nent;
  int conj;               // the op applied conj(M) (bra side of a density matrix): use conj(C)
};

int64_t layout_entries(int layout, int D);
int64_t build_scratch_entries(int gate, int D);
int gate_layout(int gate);
int launch_build_jobs(const BuildJob* d_jobs, int n_jobs, const PhaseTerm* d_terms,
                      const double* d_params, double2* arena, cudaStream_t st, int nb = 1,
                      int64_t param_stride = 0, int64_t arena_stride = 0);
int launch_param_grads(const GradOp* d_ops, const GradContrib* d_contrib, const int* d_pstart,
                       const int* d_plist, int n_params, const PhaseTerm* d_terms,
                       const double2* arena, const double2* carena, double* grads,
                       cudaStream_t st, int nb = 1, int64_t arena_stride = 0, int64_t carena_stride = 0);
