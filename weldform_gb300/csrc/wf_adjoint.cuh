// Reverse-mode (adjoint) pass of the plain FP64 kick-drift step.
//
// The adjoint runs backwards over a recomputed segment of steps.  For each
// step it reads the step's tape: the persistent state columns at the start of
// the step (after that step's neighbour search and reordering) and at its end,
// the TapeCol values of the step, the neighbour and contact rows the step used,
// and the rigid-mesh geometry of the step.  The neighbour topology is frozen
// per step: the adjoint differentiates every pair and contact term the forward
// evaluated and nothing else.
#pragma once
#include "wf_device.cuh"

namespace wf {

// Adjoint of the state carried between steps (double columns of N).
enum AdjState : int {
  A_X = 0,    // position (3)
  A_V = 3,    // velocity (3)
  A_RHO = 6,  // Density
  A_SIG = 7,  // Sigma (6), as read by the next step's acceleration pass
  A_TAU = 13, // ShearStress (6)
  A_PLS = 19, // pl_strain
  A_SY = 20,  // Sigmay
  A_T = 21,   // T
  A_DTDT = 22,// dTdt
  A_INC = 23, // Strain_pl_incr (6), read by the plastic-work heat of later steps
  NA_STATE = 29
};
// Adjoints of one step's intermediates.
enum AdjTmp : int {
  J_XN = 0,    // x(n+1) (3)
  J_VN = 3,    // v(n+1) (3)
  J_RHON = 6,  // rho(n+1)
  J_SR = 7,    // StrainRate (6)
  J_RR = 13,   // RotationRate (3)
  J_VH = 16,   // half-step velocity (3)
  J_AH = 19,   // acceleration of the second kick (3)
  J_DRHO = 22, // density rate
  J_AACC = 23, // acceleration from the pair sum (3)
  J_LC = 26,   // adjoint of dTdt(n+1) over rho(n+1) cp (the conduction sum's factor)
  NA_TMP = 27
};
// Per-particle accumulators of parameter adjoints (permuted with the state).
enum AdjParamCol : int {
  Q_G = 0,     // d loss / d G_i
  Q_CS,        // d loss / d Cs_i
  Q_SY0,       // initial Sigmay of bilinear / Hollomon particles
  Q_EP,        // Ep_i
  Q_A, Q_B, Q_N, Q_C, Q_M,  // Johnson-Cook constants
  Q_MU,        // friction coefficient (friction_sta = friction_dyn)
  Q_PFAC,      // contact stiffness factor
  NQ = 11
};
constexpr int ADJ_NPARAM = 10;  // public order: E, sy0, Ep, A, B, n, C, m, mu, PFAC
constexpr int ADJ_MAX_INSIDE = 8;  // inside contact pairs per particle in one step
constexpr int ERR_ADJ_CONTACT = 32;
constexpr int ADJ_BLOCK = 256;   // threads of the adjoint's per-particle kernels

struct AdjPtrs {
  DevPtrs S;          // start-of-step view: state, ints, rows, contact rows, mesh geometry of the step
  const double* fe;   // end-of-step persistent columns (same layout as S.f)
  const double* tx;   // the step's TapeCol columns
  const double* Lin;  // adjoint at the end of the step (AdjState)
  double* Lout;       // adjoint at the start of the step (AdjState)
  double* Tmp;        // AdjTmp
  // Pair geometry per row entry (ELL, entry k of particle i at k * N + i):
  // GradKernel and (dGK/dr)/r at the step's start positions, formed by R3 and
  // read by R4, and at its end positions, formed by R1 (thermal steps) and
  // read by R2.
  double* gk_start;
  double* dg_start;
  double* gk_end;
  double* dg_end;
  double* Q;          // AdjParamCol accumulators
  int* err;
  double time;        // Time at the start of the step (velocity-BC amplitudes)
  double seed[3];     // d loss / d (reaction force of mesh seed_mesh) of this step
  int seed_mesh;
};

void launch_adjoint_step(const AdjPtrs& A, const DomainConst& K, cudaStream_t s);
// Scatter ncol columns of src (new order) into dst (old order): dst[perm[p]] = src[p].
void launch_unpermute(const int* perm, const double* src, double* dst, int ncol, int N, cudaStream_t s);
// Adds the initial-Sigmay terms and the E chain rule, then reduces the
// accumulators to ADJ_NPARAM sums (fixed order) into out.
void launch_adjoint_finish(const DevPtrs& P0, const DomainConst& K, const double* Lstart, double* Q, double* partials,
                           double* out, cudaStream_t s);
void launch_record_force(const DevPtrs& P, int mesh, int axis, double* out, long long n, cudaStream_t s);

}  // namespace wf
