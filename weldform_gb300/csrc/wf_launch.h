// Host-side launch entry points of the device kernels (one stream per domain).
#pragma once
#include "wf_device.cuh"

namespace wf {

// Launch bookkeeping: every kernel launch of a step is followed by mark(),
// which counts launches and, during an instrumented run, records a CUDA event
// on the launching stream so each kernel's duration can be read back.
struct KernelTimer {
  cudaEvent_t* ev = nullptr;
  const char** names = nullptr;
  int cap = 0, n = 0;
};
extern thread_local KernelTimer* g_timer;
extern thread_local long long g_launches;
inline void mark(cudaStream_t s, const char* name) {
  ++g_launches;
  KernelTimer* t = g_timer;
  if (t && t->n < t->cap) {
    cudaEventRecord(t->ev[t->n], s);
    t->names[t->n] = name;
    ++t->n;
  }
}

// Conditional search in a captured step: while a step graph is captured with
// g_search_cond set, the step head asks it for a graph conditional handle,
// which k_schedule sets to the step's search decision, and captures the
// search (and the mixed form's record refresh) into the body of an IF node on
// that handle.  A step that does not search then launches none of the search
// kernels instead of launching each to return at once.  Implemented by the
// domain (it owns the streams); any failure throws and the domain captures
// the plain gated form instead.
struct SearchCond {
  virtual unsigned long long begin(cudaStream_t s) = 0;   // before k_schedule: the handle
  virtual cudaStream_t open_body(cudaStream_t s) = 0;     // after it: the stream to capture the body on
  virtual void close_body() = 0;                          // after the body's kernels
  virtual ~SearchCond() {}
};
extern thread_local SearchCond* g_search_cond;

// Neighbour search pipeline (wf_nbsearch.cu); every kernel is gated on
// StepState::do_search.
void launch_neighbour_search(const DevPtrs& P, const DomainConst& K, double* fscratch, int* iscratch,
                             cudaStream_t s);
// Halo lists and row slots of the staged mixed gathers (wf_step_mixed.cu),
// after the rows are built; gated on the search flag like the search.
void launch_halo_build(const DevPtrs& P, const DomainConst& K, cudaStream_t s);
// Shared-memory limit of the staged gathers for a halo capacity (a cudaError_t).
int configure_staging(int cap);
// Forces the search on the next launch (solver prologue and explicit calls).
void launch_force_search(const DevPtrs& P, cudaStream_t s);

// Pieces shared by both forms (wf_step_fp64.cu): schedule + gated search;
// velocity BCs on a velocity column; contact + first half kick; reductions,
// rigid-mesh update and schedule bookkeeping.
void launch_step_head(const DevPtrs& P, const DomainConst& K, double* fscratch, int* iscratch, cudaStream_t s);
void launch_bc(const DevPtrs& P, const DomainConst& K, int vcol, cudaStream_t s);
void launch_contact_kick(const DevPtrs& P, const DomainConst& K, cudaStream_t s);
void launch_step_tail(const DevPtrs& P, const DomainConst& K, cudaStream_t s);
// Float shadows of the mixed form from the FP64 state (gated on the search
// flag unless force is set).
void launch_refresh_shadows(const DevPtrs& P, const DomainConst& K, int force, cudaStream_t s);

// One kick-drift step of the plain FP64 form (wf_step_fp64.cu), and the part
// of it after the schedule and search (the adjoint's recompute snapshots the
// state between the two).
void launch_step_fp64(const DevPtrs& P, const DomainConst& K, double* fscratch, int* iscratch, cudaStream_t s);
void launch_step_fp64_body(const DevPtrs& P, const DomainConst& K, cudaStream_t s);
// Tensile-instability stress TIR of every particle (no-op unless K.ti).
void launch_tensile(const DevPtrs& P, const DomainConst& K, cudaStream_t s);
// One kick-drift step of the mixed FP32/FP64 form (wf_step_mixed.cu).
void launch_step_mixed(const DevPtrs& P, const DomainConst& K, double* fscratch, int* iscratch, cudaStream_t s);

// Prologue helpers: derived columns (Sigma/rho^2, m/rho, p/rho^2), initial
// pressure (InitialChecks, Domain.cpp:2097-2113) and max pl_strain.
void launch_prologue(const DevPtrs& P, const DomainConst& K, cudaStream_t s);
// Host-transfer helpers: scatter/gather between original and sorted order.
void launch_gather_orig(const DevPtrs& P, const DomainConst& K, const double* col, double* out_orig, int ncomp,
                        cudaStream_t s);
void launch_scatter_orig(const DevPtrs& P, const DomainConst& K, const double* in_orig, double* col, int ncomp,
                         cudaStream_t s);
// Symmetric (6 stored columns) or antisymmetric (3, anti = 1) tensor as 9 values per particle.
void launch_gather_orig_tensor(const DevPtrs& P, const DomainConst& K, const double* col, double* out_orig, int anti,
                               cudaStream_t s);
void launch_gather_orig_i32(const DevPtrs& P, const DomainConst& K, const int* col, int* out_orig, cudaStream_t s);
void launch_scatter_orig_i32(const DevPtrs& P, const DomainConst& K, const int* in_orig, int* col, cudaStream_t s);
// Recompute derived columns after a host write of state (x, v, rho, Sigma...).
void launch_refresh_derived(const DevPtrs& P, const DomainConst& K, cudaStream_t s);

}  // namespace wf
