// Plain FP64 form of one kick-drift step (Domain::SolveDiffUpdateKickDrift,
// Source/SolverKickDrift.cpp:117-393) on sm_103a.
//
// Launch sequence of one step (all on the domain's stream, no host sync):
//   k_schedule          neighbour-search decision (SolverKickDrift.cpp:153-186)
//   [search pipeline]   gated on the decision (wf_nbsearch.cu)
//   k_accel             CalcAccel + AccelReduction (InteractionAlt.cpp:12-260)
//   k_bc                GeneralAfter (WeldForm.cpp:51-120)
//   k_contact_kick      CalcContactForcesWang (Contact_Wang.cpp:15-348) + v += a dt/2
//   k_bc
//   k_density_drift     CalcDensInc + DensReduction (InteractionAlt.cpp:483-640) with the
//                       acceleration pass's GradKernel per row entry (same x(n), h),
//                       rho += dt drho, x += v dt, v += a dt/2 (SolverKickDrift.cpp:236-265);
//                       next-step p/rho^2 and T for the rate gather
//   k_bc                (on the next-step velocity buffer)
//   k_rate_stress       CalcRateTensors + RateTensorsReduction (InteractionAlt.cpp:263-479),
//                       CalcStressStrain (Particle.cpp:960-1067), CalcPlasticWorkHeat
//                       (ThermalStuct.cpp:14-39), T += dt dTdt (Thermal.cpp:727-734),
//                       and in the same neighbour loop CalcTempInc (Thermal.cpp:53-219),
//                       CalcKinEnergyEqn (Domain.cpp:1752-1808); then CalcThermalExpStrainRate
//                       and CalcIntEnergyEqn (Domain.cpp:1810-1829)
//   k_finalize          deterministic reduction of the per-block partial sums
//   k_mesh_*            TriMesh::Update (Mesh.cpp:273-293), UpdateContactParticles
//                       (Contact.cpp:41-55)
//   k_step_end          Time += dt and the neighbour-clear schedule (:299-324)
//
// Each gather kernel runs one thread per particle over its neighbour row in
// canonical order; a pair term is evaluated from the particle's own side
// (x_i - x_j), which equals the reference's (min, max)-ordered pair value
// with the reduction's sign applied.
#include "wf_step_common.cuh"
#include "wf_launch.h"

namespace wf {

thread_local KernelTimer* g_timer = nullptr;
thread_local long long g_launches = 0;
thread_local SearchCond* g_search_cond = nullptr;

static inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

// ---------------------------------------------------------------- schedule
// One block.  A batched domain decides per specimen (the same rules on the
// specimen's own state) and searches when any specimen asks.  cond: the
// captured step's conditional handle of the search (0 outside such a graph).
__global__ void k_schedule(DevPtrs P, DomainConst K, unsigned long long cond) {
  StepState* s = P.st;
  __shared__ int any_search, any_regular;
  if (threadIdx.x == 0) { any_search = 0; any_regular = 0; }
  __syncthreads();
  for (int q = threadIdx.x; q < K.nspec; q += blockDim.x) {
    SpecState& sp = P.sp[q];
    sp.yielded = sp.yielded_next;
    int search = 0, regular = 0;
    if (sp.yielded && !sp.isyielding) {
      search = 1;
      sp.isyielding = 1;
    } else if ((sp.yielded || s->isfirst) && sp.ts_i == 0 && sp.nb_cleared) {
      search = 1;
      regular = 1;
    }
    if (K.freeze_nb && !s->isfirst) search = regular = 0;
    if (search) { sp.nb_cleared = 0; sp.searches += 1; atomicOr(&any_search, 1); }
    if (regular) atomicOr(&any_regular, 1);
    sp.do_search = search;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  double mx = s->max_pl_next;
  s->max_pl = mx;
  int search = 0, regular = 0;
  if (mx > MIN_PS_FOR_NBSEARCH && !s->isyielding) {  // first yield
    search = 1;
    s->isyielding = 1;
  } else if ((mx > MIN_PS_FOR_NBSEARCH || s->isfirst) && s->ts_i == 0 && s->nb_cleared) {
    search = 1;
    regular = 1;
  }
  // Frozen topology (a library option for finite-difference checks of the
  // adjoint, which differentiates each step with its topology fixed): after
  // the first step's search the rows, contact pairs and surface flags stay.
  if (K.freeze_nb && !s->isfirst) search = regular = 0;
  if (K.nspec > 0) { search = any_search; regular = any_regular; }
  if (search) s->nb_cleared = 0;
  s->do_search = search;
  // CalcGradCorrMatrix: kick-drift at its first step (SolverKickDrift.cpp:189-191),
  // leapfrog after every regular search and at the first step (SolverLeapfrog.cpp:186-204)
  s->do_gradcorr = K.gradcorr && (s->isfirst || (K.leapfrog && regular));
  if (cond) cudaGraphSetConditional((cudaGraphConditionalHandle)cond, search ? 1u : 0u);
}

__global__ void k_step_end(DevPtrs P, DomainConst K) {
  StepState* s = P.st;
  for (int q = threadIdx.x; q < K.nspec; q += blockDim.x) {  // each specimen's own cadence
    SpecState& sp = P.sp[q];
    if (sp.yielded) {
      if (sp.ts_i == (K.ts_nb_inc - 1)) sp.nb_cleared = 1;
      sp.ts_i++;
      if (sp.ts_i > (K.ts_nb_inc - 1)) sp.ts_i = 0;
    }
    sp.do_search = 0;
  }
  if (threadIdx.x != 0) return;
  s->gk_valid = K.mixed ? 0 : 1;  // the plain rate pass left GradKernel at the new positions
  s->steps += 1;
  s->Time += s->deltat;
  s->isfirst = 0;
  if (s->max_pl > MIN_PS_FOR_NBSEARCH) {
    if (s->ts_i == (K.ts_nb_inc - 1)) s->nb_cleared = 1;
    s->ts_i++;
    if (s->ts_i > (K.ts_nb_inc - 1)) s->ts_i = 0;
  }
  s->do_search = 0;
}

// ---------------------------------------------------------------- geometry
struct PairGeo {
  double x0, x1, x2;  // x_i - x_j
  double r2, r, hh, GK;
};
// Pair geometry: h = (hi + hj) / 2, q = rij / h, cubic-spline GradKernel
// (Functions.cpp:74-87), C = 1 / (pi h^4):
//   q < 1:      GK = C/h (-3 + 9/4 q)
//   1 <= q < 2: GK = -3/4 C (2 - q)^2 / (q h) = -3/4 C (2 - q)^2 / r
// GB300 runs FP64 division as a multi-instruction sequence at 1/64 of the
// FP32 rate, so the pair takes one division (C / r, only for q >= 1) plus
// 1/h when the two smoothing lengths differ; inv_hi = 1/h_i comes from the
// caller.  Equal to the reference's expression to rounding.
__device__ __forceinline__ PairGeo pair_geo(double xi0, double xi1, double xi2, double hi, double inv_hi, double xj0,
                                           double xj1, double xj2, double hj) {
  PairGeo g;
  g.x0 = xi0 - xj0; g.x1 = xi1 - xj1; g.x2 = xi2 - xj2;
  g.r2 = g.x0 * g.x0 + g.x1 * g.x1 + g.x2 * g.x2;
  // r and 1/r from one reciprocal square root instead of a square root and a
  // division (r2 = 0 only for coincident particles, where q = 0)
  double ir = g.r2 > 0.0 ? rsqrt(g.r2) : 0.0;
  g.r = g.r2 * ir;
  double inv_h;
  if (hj == hi) { g.hh = hi; inv_h = inv_hi; }
  else { g.hh = (hi + hj) / 2; inv_h = 1.0 / g.hh; }
  double q = g.r * inv_h;
  double ih2 = inv_h * inv_h;
  double C = ih2 * ih2 * (1.0 / WF_PI);
  if (q == 0.0) g.GK = C * inv_h * -3.0;
  else if (q < 1.0) g.GK = C * inv_h * (-3.0 + 2.25 * q);
  else if (q < 2.0) { double t = 2.0 - q; g.GK = C * ir * (-0.75 * t * t); }
  else g.GK = 0.0;
  return g;
}

// ---------------------------------------------------------------- tensile instability
// StartAcceleration's TIR (Domain.cpp:1557-1569): TIR = V diag(f(L)) V^T for
// the eigen-decomposition of Sigma, f(l) = -TI l / rho^2 for l > 0, else 0;
// products summed k = 2, 1, 0 as matvec.h's Mult.  The mixed form, whose pair
// terms read TIR in FP32, decomposes in FP32 (eig_sym3f): the FP64 Jacobi
// sweeps' square roots and divisions would cost it more than its whole step
// at 1M particles.  Also fills the mixed form's FP32 groups.
__global__ void k_tensile(DevPtrs P, DomainConst K) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K.N) return;
  size_t N = K.N;
  double tir[6] = {0, 0, 0, 0, 0, 0};
  double ti = col(P, C_TI, N, i);
  const int ui[6] = {0, 1, 2, 0, 0, 1}, uj[6] = {0, 1, 2, 1, 2, 2};
  if (icol(P, I_KIND, N, i) == 0 && ti > 0.0) {
    double rho = col(P, C_RHO, N, i);
    double rho2 = rho * rho;
    double pc = ti / (rho2);
    if (K.mixed) {
      float sg[6], L[3], V[3][3], f[3];
      for (int c = 0; c < 6; ++c) sg[c] = (float)col(P, C_SIG + c, N, i);
      eig_sym3f(sg, L, V);
      for (int k = 0; k < 3; ++k) f[k] = (L[k] > 0.0f) ? -(float)pc * L[k] : 0.0f;
      for (int c = 0; c < 6; ++c) {
        int a = ui[c], b = uj[c];
        tir[c] = (double)((V[a][2] * f[2]) * V[b][2] + (V[a][1] * f[1]) * V[b][1] + (V[a][0] * f[0]) * V[b][0]);
      }
    } else {
      double sg[6], L[3], V[3][3];
      for (int c = 0; c < 6; ++c) sg[c] = col(P, C_SIG + c, N, i);
      eig_sym3(sg, L, V);
      double f[3];
      for (int k = 0; k < 3; ++k) f[k] = (L[k] > 0) ? -pc * L[k] : 0.0;
      for (int c = 0; c < 6; ++c) {
        int a = ui[c], b = uj[c];
        tir[c] = (V[a][2] * f[2]) * V[b][2] + (V[a][1] * f[1]) * V[b][1] + (V[a][0] * f[0]) * V[b][0];
      }
    }
  }
  for (int c = 0; c < 6; ++c) colw(P, C_TIR + c, N, i) = tir[c];
  if (K.mixed) {
    P.rc[(size_t)RC_TI0 * N + i] = make_float4((float)tir[0], (float)tir[1], (float)tir[2], (float)tir[3]);
    P.rc[(size_t)RC_TI1 * N + i] =
        make_float4((float)tir[4], (float)tir[5], (float)col(P, C_TIN, N, i), (float)col(P, C_TIDIST, N, i));
  }
}

// ---------------------------------------------------------------- kernel-gradient correction
// Domain::CalcGradCorrMatrix (Domain.cpp:1832-1940): M_i = -sum_j (m_j/rho_j)
// (GK x_ij) (x) x_ij over the particle's row, gradCorrM = InvLog(M_i)
// (matvec.h:673-693; the identity when |det| < 1e-10).  The dyad is even in
// x_ij, so each end's own x_i - x_j gives the reference's value.
__global__ void k_grad_corr(DevPtrs P, DomainConst K) {
  if (!P.st->do_gradcorr) return;
  size_t N = K.N;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K.N; i += gridDim.x * blockDim.x) {
    if (icol(P, I_KIND, N, i) != 0) continue;
    double xi0 = col(P, C_X, N, i), xi1 = col(P, C_X + 1, N, i), xi2 = col(P, C_X + 2, N, i), hi = col(P, C_H, N, i);
    double inv_hi = 1.0 / hi;
    double t[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    int len = P.row_len[i];
    for (int k = 0; k < len; ++k) {
      int j = nb_index(P.nbr[(size_t)k * N + i]);
      PairGeo g = pair_geo(xi0, xi1, xi2, hi, inv_hi, col(P, C_X, N, j), col(P, C_X + 1, N, j), col(P, C_X + 2, N, j),
                           col(P, C_H, N, j));
      double gv[3] = {g.GK * g.x0, g.GK * g.x1, g.GK * g.x2}, xv[3] = {g.x0, g.x1, g.x2};
      double f = col(P, C_MASS, N, j) / col(P, C_RHO, N, j);
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) t[3 * a + b] = t[3 * a + b] - f * (gv[a] * xv[b]);
    }
    double det = t[0] * (t[4] * t[8] - t[5] * t[7]) - t[1] * (t[3] * t[8] - t[5] * t[6]) +
                 t[2] * (t[3] * t[7] - t[4] * t[6]);
    double m[9];
    if (fabs(det) < 1.0e-10) {
      for (int c = 0; c < 9; ++c) m[c] = (c % 4 == 0) ? 1.0 : 0.0;
    } else {
      m[0] = (t[4] * t[8] - t[5] * t[7]) / det; m[1] = (t[2] * t[7] - t[1] * t[8]) / det; m[2] = (t[1] * t[5] - t[2] * t[4]) / det;
      m[3] = (t[5] * t[6] - t[3] * t[8]) / det; m[4] = (t[0] * t[8] - t[2] * t[6]) / det; m[5] = (t[2] * t[3] - t[0] * t[5]) / det;
      m[6] = (t[3] * t[7] - t[4] * t[6]) / det; m[7] = (t[1] * t[6] - t[0] * t[7]) / det; m[8] = (t[0] * t[4] - t[1] * t[3]) / det;
    }
    for (int c = 0; c < 9; ++c) colw(P, C_GCM + c, N, i) = m[c];
  }
}
// Corrected gradient Mult(GK * gradCorrM_i, x) (InteractionAlt.cpp:114-132).
__device__ __forceinline__ void corr_grad(const DevPtrs& P, size_t N, int i, double GK, double x0, double x1,
                                          double x2, double out[3]) {
  for (int k = 0; k < 3; ++k)
    out[k] = x0 * (GK * col(P, C_GCM + 3 * k, N, i)) + x1 * (GK * col(P, C_GCM + 3 * k + 1, N, i)) +
             x2 * (GK * col(P, C_GCM + 3 * k + 2, N, i));
}

// ---------------------------------------------------------------- accel
__global__ void __launch_bounds__(BLOCK) k_accel(DevPtrs P, DomainConst K) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K.N) return;
  size_t N = K.N;
  if (icol(P, I_KIND, N, i) != 0) {  // StartAcceleration resets a for every particle
    colw(P, C_A, N, i) = 0.0; colw(P, C_A + 1, N, i) = 0.0; colw(P, C_A + 2, N, i) = 0.0;
    return;
  }
  double xi0 = col(P, C_X, N, i), xi1 = col(P, C_X + 1, N, i), xi2 = col(P, C_X + 2, N, i);
  double vi0 = col(P, C_V, N, i), vi1 = col(P, C_V + 1, N, i), vi2 = col(P, C_V + 2, N, i);
  double hi = col(P, C_H, N, i), rhoi = col(P, C_RHO, N, i), csi = col(P, C_CS, N, i);
  double inv_hi = 1.0 / hi;
  double ai = col(P, C_ALPHA, N, i), bi = col(P, C_BETA, N, i);
  double tii = K.ti ? col(P, C_TI, N, i) : 0.0;
  double Si[6];
  for (int c = 0; c < 6; ++c) Si[c] = col(P, C_SRHO + c, N, i);
  double a0 = 0, a1 = 0, a2 = 0;
  int len = P.row_len[i];
  // The last step's rate pass formed GradKernel at these positions and rows
  // unless this step searched (or the host touched the state).
  const bool reuse = P.st->gk_valid && !P.st->do_search;
  for (int k = 0; k < len; ++k) {
    int j = nb_index(P.nbr[(size_t)k * N + i]);
    PairGeo g;
    if (reuse) {
      double hj = col(P, C_H, N, j);
      g.x0 = xi0 - col(P, C_X, N, j); g.x1 = xi1 - col(P, C_X + 1, N, j); g.x2 = xi2 - col(P, C_X + 2, N, j);
      g.r2 = g.x0 * g.x0 + g.x1 * g.x1 + g.x2 * g.x2;
      g.hh = hj == hi ? hi : (hi + hj) / 2;
      g.r = K.ti ? sqrt(g.r2) : 0.0;  // the tensile term alone needs r
      g.GK = P.gk[(size_t)k * N + i];
    } else {
      g = pair_geo(xi0, xi1, xi2, hi, inv_hi, col(P, C_X, N, j), col(P, C_X + 1, N, j), col(P, C_X + 2, N, j),
                   col(P, C_H, N, j));
      P.gk[(size_t)k * N + i] = g.GK;  // for the density pass (same x(n), h)
    }
    // (a + a) / 2 = a exactly, so uniform constants need no per-pair loads
    double Alpha = K.av_uniform ? ai : (ai + col(P, C_ALPHA, N, j)) / 2.0;
    double Beta = K.av_uniform ? bi : (bi + col(P, C_BETA, N, j)) / 2.0;
    double v0 = vi0 - col(P, C_V, N, j), v1 = vi1 - col(P, C_V + 1, N, j), v2 = vi2 - col(P, C_V + 2, N, j);
    double PIs = 0.0;
    if (Alpha != 0.0 || Beta != 0.0) {
      double dvx = v0 * g.x0 + v1 * g.x1 + v2 * g.x2;
      if (dvx < 0) {  // MU = h dvx / Dn, PIs = (Alpha Cij MU + Beta MU^2) / rho_bar in one division
        double Dn = g.r2 + 0.01 * g.hh * g.hh;
        double hv = g.hh * dvx;
        double Cij = 0.5 * (csi + col(P, C_CS, N, j));
        PIs = hv * (Alpha * Cij * Dn + Beta * hv) / (Dn * Dn * (0.5 * (rhoi + col(P, C_RHO, N, j))));
      }
    }
    double S0 = Si[0] + col(P, C_SRHO + 0, N, j) + PIs;
    double S1 = Si[1] + col(P, C_SRHO + 1, N, j) + PIs;
    double S2 = Si[2] + col(P, C_SRHO + 2, N, j) + PIs;
    double S3 = Si[3] + col(P, C_SRHO + 3, N, j);
    double S4 = Si[4] + col(P, C_SRHO + 4, N, j);
    double S5 = Si[5] + col(P, C_SRHO + 5, N, j);
    if (K.ti && (tii > 0.0 || col(P, C_TI, N, j) > 0.0)) {
      // TIij = (W(rij/h) / W(dinit/h))^((n_i + n_j)/2) (TIR_i + TIR_j) (InteractionAlt.cpp:102-109)
      double q0 = (col(P, C_TIDIST, N, i) + col(P, C_TIDIST, N, j)) / (2.0 * g.hh);
      double fb = kernel_shape(g.r / g.hh) / kernel_shape(q0), fn = (col(P, C_TIN, N, i) + col(P, C_TIN, N, j)) / 2.0;
      double f;
      if (fn == 4.0) { f = fb * fb; f = f * f; }  // the JSON driver's TIn: two products, not FP64 pow's log and exp
      else f = pow(fb, fn);
      S0 = S0 + f * (col(P, C_TIR + 0, N, i) + col(P, C_TIR + 0, N, j));
      S1 = S1 + f * (col(P, C_TIR + 1, N, i) + col(P, C_TIR + 1, N, j));
      S2 = S2 + f * (col(P, C_TIR + 2, N, i) + col(P, C_TIR + 2, N, j));
      S3 = S3 + f * (col(P, C_TIR + 3, N, i) + col(P, C_TIR + 3, N, j));
      S4 = S4 + f * (col(P, C_TIR + 4, N, i) + col(P, C_TIR + 4, N, j));
      S5 = S5 + f * (col(P, C_TIR + 5, N, i) + col(P, C_TIR + 5, N, j));
    }
    double mj = col(P, C_MASS, N, j);
    double g0, g1, g2;
    if (K.gradcorr) {  // temp_c = Mult(vc_i, S) of the locking sum (InteractionAlt.cpp:166-170)
      double vc[3];
      corr_grad(P, N, i, g.GK, g.x0, g.x1, g.x2, vc);
      g0 = mj * vc[0]; g1 = mj * vc[1]; g2 = mj * vc[2];
    } else {
      double gm = mj * g.GK;  // m_j (GK x_ij) . S
      g0 = gm * g.x0; g1 = gm * g.x1; g2 = gm * g.x2;
    }
    a0 += g0 * S0 + g1 * S3 + g2 * S4;
    a1 += g0 * S3 + g1 * S1 + g2 * S5;
    a2 += g0 * S4 + g1 * S5 + g2 * S2;
  }
  colw(P, C_A, N, i) = a0; colw(P, C_A + 1, N, i) = a1; colw(P, C_A + 2, N, i) = a2;
}

// ---------------------------------------------------------------- BCs
// GeneralAfter: particles whose ID matches a velocity BC get a = 0 and
// v = value (constant or amplitude); rigid meshes with that id get m_v.
__global__ void k_bc(DevPtrs P, DomainConst K, int vcol) {
  const DomainTables* T = P.tab;
  double t = P.st->Time;
  if (blockIdx.x == 0 && threadIdx.x == 0 && K.contact) {
    for (int b = 0; b < T->nbc; ++b)
      for (int m = 0; m < K.nmeshes; ++m)
        if (K.contact_surf_id[m] == T->bc[b].zone) {
          if (T->bc[b].value_type == 0) {
            for (int d = 0; d < 3; ++d) { P.st->mesh_v[m][d] = T->bc[b].value[d]; P.st->mesh_w[m][d] = T->bc[b].value_ang[d]; }
          } else {
            bool found = false;
            double val = T->bc[b].amp_factor * amp_value(T, T->bc[b].amp_id, t, &found);
            if (found) for (int d = 0; d < 3; ++d) P.st->mesh_v[m][d] = val * T->bc[b].value[d];
          }
        }
  }
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K.nbc_particles) return;
  size_t N = K.N;
  int i = P.inv[P.bc_list[k]];
  double vb[3];
  if (bc_velocity(T, icol(P, I_ID, N, i), t, vb))
    for (int d = 0; d < 3; ++d) { colw(P, C_A + d, N, i) = 0.0; colw(P, vcol + d, N, i) = vb[d]; }
  if (K.mixed)  // keep the float-float velocity in the records in step with the FP64 value
    for (int d = 0; d < 3; ++d) rec_set_v(P, N, i, d, col(P, vcol + d, N, i), vcol == C_VN);
}

// ---------------------------------------------------------------- contact + kick
__device__ __forceinline__ double dot3(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
__device__ __forceinline__ double norm3(const double a[3]) { return sqrt(dot3(a, a)); }

// NM: per-mesh force accumulators a thread keeps — 0 without contact, 1 with
// one rigid mesh (kept in registers), MAX_MESHES with several (indexed by the
// pair's mesh, so they live in local memory).
template <int NM>
__global__ void __launch_bounds__(BLOCK) k_contact_kick(DevPtrs P, DomainConst K) {
  __shared__ double sh[32];
  constexpr bool CONTACT = NM > 0;
  constexpr int NV = NM > 0 ? NM : 1;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  size_t N = K.N;
  double dt = P.st->deltat;  // the step's time step before AdaptiveTimeStep (prev_deltat)
  double cfsum = 0, crsum = 0, extw = 0;
  unsigned ndyn = 0;       // pairs of this thread in the dynamic-friction branch
  double dta = 1.0 / 0.0;  // CheckMinTSAccel candidate (kick-drift, after contact)
  double cfv[NV][3];
  for (int m = 0; m < NV; ++m) cfv[m][0] = cfv[m][1] = cfv[m][2] = 0.0;
  if (i < K.N) {
    int kind = icol(P, I_KIND, N, i);
    double a[3] = {col(P, C_A, N, i), col(P, C_A + 1, N, i), col(P, C_A + 2, N, i)};
    if (P.tx)
      for (int d = 0; d < 3; ++d) P.tx[(size_t)(TX_APRE + d) * N + i] = a[d];
    if (CONTACT) {
      double cf[3] = {0, 0, 0}, dcont = 0.0;
      int ncp = kind == 0 ? P.cp_len[i] : 0;
      if (ncp > 0) {
        double x[3] = {col(P, C_X, N, i), col(P, C_X + 1, N, i), col(P, C_X + 2, N, i)};
        double v[3] = {col(P, C_V, N, i), col(P, C_V + 1, N, i), col(P, C_V + 2, N, i)};
        double m1 = col(P, C_MASS, N, i), h1 = col(P, C_H, N, i);
        for (int k = 0; k < ncp; ++k) {
          int p2 = P.cp[(size_t)k * N + i];
          double n2[3] = {col(P, C_NORMAL, N, p2), col(P, C_NORMAL + 1, N, p2), col(P, C_NORMAL + 2, N, p2)};
          double v2[3] = {col(P, C_V, N, p2), col(P, C_V + 1, N, p2), col(P, C_V + 2, N, p2)};
          double vr[3] = {v[0] - v2[0], v[1] - v2[1], v[2] - v2[2]};
          double delta_ = -dot3(n2, vr);
          int e = icol(P, I_ELEM, N, p2);
          int m = icol(P, I_MESH, N, p2);
          double xp[3];
          for (int d = 0; d < 3; ++d) xp[d] = x[d] + v[d] * dt + a[d] * dt * dt / 2.0;
          double dist = dot3(n2, xp) - P.elem_pplane[e];
          if (!(dist < h1)) continue;
          double qj[3] = {x[0] - dist * n2[0], x[1] - dist * n2[1], x[2] - dist * n2[2]};
          bool inside = true;
          for (int ii = 0; ii < 3 && inside; ++ii) {
            int jj = ii + 1; if (jj > 2) jj = 0;
            int na = P.elem_node[3 * e + ii], nb = P.elem_node[3 * e + jj];
            double pa[3] = {P.node[na], P.node[P.nnodes + na], P.node[2 * P.nnodes + na]};
            double pb[3] = {P.node[nb], P.node[P.nnodes + nb], P.node[2 * P.nnodes + nb]};
            double u[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
            double w[3] = {qj[0] - pa[0], qj[1] - pa[1], qj[2] - pa[2]};
            double c[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
            if (dot3(c, n2) < 0.0) inside = false;
          }
          if (!inside) continue;
          double delta = h1 - dist;
          double kij;
          if (K.contact_alg == 1) {
            double rho1 = col(P, C_RHO0, N, i), cs = col(P, C_CS, N, i), G = col(P, C_G, N, i);
            double bulk = cs * cs * rho1;
            double dS = pow(m1 / rho1, 0.33333);
            kij = K.PFAC * (9. * bulk * G / (3. * bulk + G) * dS);
          } else if (K.contact_alg == 2) {
            kij = K.PFAC * pow(m1 / col(P, C_RHO, N, i), 2.0 / 3.0);
          } else {
            kij = 2.0 * m1 / (dt * dt);
          }
          double omega = sqrt(kij / m1);
          double psi = 2. * m1 * omega * K.DFAC;
          double s = kij * delta - psi * delta_;
          for (int d = 0; d < 3; ++d) cf[d] = s * n2[d];
          dcont = delta;
          for (int d = 0; d < 3; ++d) a[d] = a[d] + cf[d] / m1;
          if (K.friction_sta > 0.) {
            double du[3];
            for (int d = 0; d < 3; ++d) du[d] = (xp[d] - x[d]) - v2[d] * dt;
            double dn = dot3(du, n2);
            double tg[3];
            for (int d = 0; d < 3; ++d) tg[d] = kij * (du[d] - dn * n2[d]);
            double ntg = norm3(tg), ncf = norm3(cf);
            if (ntg < K.friction_sta * ncf) {
              for (int d = 0; d < 3; ++d) { double q = tg[d] / m1; cf[d] -= q; a[d] -= q; }
            } else {  // dynamic branch (Contact_Wang.cpp:284-290)
              ++ndyn;
              double fs = K.friction_dyn * ncf;
              for (int d = 0; d < 3; ++d) { double td = fs * tg[d] / ntg; cf[d] -= td; a[d] -= td / m1; }
            }
          }
          cfsum += norm3(cf);
          if (NM == 1) for (int d = 0; d < 3; ++d) cfv[0][d] += cf[d];  // the only mesh
          else if (m < NV) for (int d = 0; d < 3; ++d) cfv[m][d] += cf[d];
          crsum += dot3(a, n2) * m1;
          extw += dot3(cf, v2);
        }
      }
      for (int d = 0; d < 3; ++d) colw(P, C_CF + d, N, i) = cf[d];
      colw(P, C_DCONT, N, i) = dcont;
      for (int d = 0; d < 3; ++d) colw(P, C_A + d, N, i) = a[d];
    }
    if (K.auto_ts_acc && !K.leapfrog)  // Domain.cpp:309
      dta = K.sqrt_h_a * sqrt(col(P, C_H, N, i) / sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]));
    if (K.leapfrog) {  // first leapfrog step starts from v - a dt/2 (SolverLeapfrog.cpp:233-236)
      if (P.st->isfirst)
        for (int d = 0; d < 3; ++d) {
          double vn = col(P, C_V + d, N, i) - a[d] * 0.5 * dt;
          colw(P, C_V + d, N, i) = vn;
          if (K.mixed) rec_set_v(P, N, i, d, vn, false);
        }
    } else if (kind == 0) {  // half kick v += a * 0.5 * dt (rigid-mesh particles have a = 0)
      double vn[3];
      for (int d = 0; d < 3; ++d) {
        vn[d] = col(P, C_V + d, N, i) + a[d] * 0.5 * dt;
        colw(P, C_V + d, N, i) = vn[d];
      }
      if (K.mixed) rec_set_v3(P, N, i, vn);
    }
    // GeneralAfter after the kick (SolverKickDrift.cpp:231) on this particle,
    // in place of a BC pass: it depends on no other particle, and a rigid-mesh
    // particle another thread reads here keeps the velocity the pass before
    // the contact gave it.
    double vb[3];
    if (!K.leapfrog && bc_velocity(P.tab, icol(P, I_ID, N, i), P.st->Time, vb)) {
      for (int d = 0; d < 3; ++d) { colw(P, C_A + d, N, i) = 0.0; colw(P, C_V + d, N, i) = vb[d]; }
      if (K.mixed) rec_set_v3(P, N, i, vb);
    }
  }
  if (K.auto_ts_acc && !K.leapfrog) {
    double r = block_reduce<2>(dta, sh);
    if (threadIdx.x == 0) P.partials[S_DTA * K.nblocks + blockIdx.x] = r;
  }
  if (CONTACT) {
    // one counter update per warp (a per-pair atomic on one address serialised
    // the kernel on contact-heavy steps)
    unsigned wdyn = __reduce_add_sync(0xffffffffu, ndyn);
    if ((threadIdx.x & 31) == 0 && wdyn) atomicAdd(&P.st->dyn_friction, (unsigned long long)wdyn);
    double r;
    r = block_reduce<0>(cfsum, sh); if (threadIdx.x == 0) P.partials[S_CFSUM * K.nblocks + blockIdx.x] = r;
    r = block_reduce<0>(crsum, sh); if (threadIdx.x == 0) P.partials[S_CRSUM * K.nblocks + blockIdx.x] = r;
    r = block_reduce<0>(extw, sh); if (threadIdx.x == 0) P.partials[S_EXTW * K.nblocks + blockIdx.x] = r;
    for (int m = 0; m < K.nmeshes && m < NV; ++m)
      for (int d = 0; d < 3; ++d) {
        r = block_reduce<0>(cfv[m][d], sh);
        if (threadIdx.x == 0) P.partials[(S_CFVEC + 3 * m + d) * K.nblocks + blockIdx.x] = r;
      }
  }
}

// ---------------------------------------------------------------- density + drift + kick
__global__ void __launch_bounds__(BLOCK) k_density_drift(DevPtrs P, DomainConst K) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K.N) return;
  size_t N = K.N;
  double dt = P.st->deltat;
  double xi0 = col(P, C_X, N, i), xi1 = col(P, C_X + 1, N, i), xi2 = col(P, C_X + 2, N, i);
  double vi0 = col(P, C_V, N, i), vi1 = col(P, C_V + 1, N, i), vi2 = col(P, C_V + 2, N, i);
  double rhoi = col(P, C_RHO, N, i);
  double dd = 0.0;
  if (P.tx) {
    P.tx[(size_t)(TX_VH + 0) * N + i] = vi0; P.tx[(size_t)(TX_VH + 1) * N + i] = vi1;
    P.tx[(size_t)(TX_VH + 2) * N + i] = vi2;
  }
  if (icol(P, I_KIND, N, i) == 0) {
    int len = P.row_len[i];
    for (int k = 0; k < len; ++k) {
      int j = nb_index(P.nbr[(size_t)k * N + i]);
      // x(n) and h are the acceleration pass's: its GradKernel of this entry is reused
      PairGeo g;
      g.x0 = xi0 - col(P, C_X, N, j); g.x1 = xi1 - col(P, C_X + 1, N, j); g.x2 = xi2 - col(P, C_X + 2, N, j);
      g.GK = P.gk[(size_t)k * N + i];
      double v0 = vi0 - col(P, C_V, N, j), v1 = vi1 - col(P, C_V + 1, N, j), v2 = vi2 - col(P, C_V + 2, N, j);
      if (K.gradcorr) {  // locking form m_j (rho_i/rho_j) v_ij . vc_i (InteractionAlt.cpp:589-605)
        double vc[3];
        corr_grad(P, N, i, g.GK, g.x0, g.x1, g.x2, vc);
        double t1 = v0 * vc[0] + v1 * vc[1] + v2 * vc[2];
        dd += col(P, C_MASS, N, j) * (rhoi / col(P, C_RHO, N, j)) * t1;
        continue;
      }
      double pd = v0 * (g.GK * g.x0) + v1 * (g.GK * g.x1) + v2 * (g.GK * g.x2);
      dd += col(P, C_MRHO, N, j) * pd;
    }
    if (!K.gradcorr) dd *= rhoi;
  }
  colw(P, C_DRHO, N, i) = dd;
  double rn = rhoi + dt * dd;
  colw(P, C_RHON, N, i) = rn;
  colw(P, C_MRHON, N, i) = icol(P, I_KIND, N, i) == 0 ? col(P, C_MASS, N, i) / rn : 0.0;
  // Next-step pressure over density^2 (EOS case 0 of the updated density, the
  // expression the stress update evaluates) and next-step temperature
  // (Thermal.cpp:727-734): the fused rate gather reads both for neighbours.
  {
    double cs = col(P, C_CS, N, i);
    double pn = col(P, C_P0, N, i) + (cs * cs) * (rn - col(P, C_RHO0, N, i));
    colw(P, C_PR2N, N, i) = pn / (rn * rn);
    if (K.thermal_solver) colw(P, C_TN, N, i) = col(P, C_T, N, i) + dt * col(P, C_DTDT, N, i);
  }
  double v[3] = {vi0, vi1, vi2}, x[3] = {xi0, xi1, xi2};
  // GeneralAfter on the next-step velocity (SolverKickDrift.cpp:267) applied
  // here instead of in a BC pass after this kernel
  double vb[3];
  const bool bc = bc_velocity(P.tab, icol(P, I_ID, N, i), P.st->Time, vb);
  for (int d = 0; d < 3; ++d) {
    double du = v[d] * dt;
    colw(P, C_DISP + d, N, i) = col(P, C_DISP + d, N, i) + du;
    colw(P, C_XN + d, N, i) = x[d] + du;
    colw(P, C_VN + d, N, i) = bc ? vb[d] : (K.leapfrog ? v[d] : v[d] + col(P, C_A + d, N, i) * dt / 2.);
    if (bc) colw(P, C_A + d, N, i) = 0.0;
  }
}

// Leapfrog kick v(n+1/2) = v(n-1/2) + a (dt_prev + dt)/2 for every particle
// (SolverLeapfrog.cpp:264-270).
__global__ void k_kick_leapfrog(DevPtrs P, DomainConst K) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K.N) return;
  size_t N = K.N;
  double f = 0.5 * (P.st->prev_deltat + P.st->deltat);
  for (int d = 0; d < 3; ++d) {
    double vn = col(P, C_V + d, N, i) + col(P, C_A + d, N, i) * f;
    colw(P, C_V + d, N, i) = vn;
    if (K.mixed) rec_set_v(P, N, i, d, vn, false);
  }
}

// ---------------------------------------------------------------- rate + stress
__global__ void __launch_bounds__(BLOCK) k_rate_stress(DevPtrs P, DomainConst K) {
  __shared__ double sh[32];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  size_t N = K.N;
  double dt = P.st->deltat;
  double plw = 0.0, maxpl = 0.0, maxT = -1e300, minT = 1e300, dkin_b = 0.0, dint = 0.0;
  if (i < K.N) {
    // Next-step buffers become the current state for this particle.
    double x[3], v[3];
    for (int d = 0; d < 3; ++d) { x[d] = col(P, C_XN + d, N, i); v[d] = col(P, C_VN + d, N, i); }
    double rho = col(P, C_RHON, N, i);
    for (int d = 0; d < 3; ++d) { colw(P, C_X + d, N, i) = x[d]; colw(P, C_V + d, N, i) = v[d]; }
    colw(P, C_RHO, N, i) = rho;
    colw(P, C_MRHO, N, i) = col(P, C_MRHON, N, i);
    maxpl = col(P, C_PLS, N, i);
    if (icol(P, I_KIND, N, i) == 0) {
      double hi = col(P, C_H, N, i);
      double inv_hi = 1.0 / hi;
      double sr[6] = {0, 0, 0, 0, 0, 0}, rr[3] = {0, 0, 0};
      // CalcKinEnergyEqn and CalcTempInc pair sums, on the same positions and
      // velocities as the rates (Domain.cpp:1752-1808, Thermal.cpp:53-219)
      double dkin = 0.0, cond = 0.0;
      double massi = col(P, C_MASS, N, i), mrhoi = col(P, C_MRHON, N, i), pri = col(P, C_PR2N, N, i);
      double Ti = 0.0, ki = 0.0;
      if (K.thermal_solver) { Ti = col(P, C_TN, N, i); ki = col(P, C_KT, N, i); }
      int len = P.row_len[i];
      for (int k = 0; k < len; ++k) {
        int e = P.nbr[(size_t)k * N + i];
        int j = nb_index(e);
        PairGeo g = pair_geo(x[0], x[1], x[2], hi, inv_hi, col(P, C_XN, N, j), col(P, C_XN + 1, N, j), col(P, C_XN + 2, N, j),
                             col(P, C_H, N, j));
        P.gk[(size_t)k * N + i] = g.GK;  // x(n+1) is the next step's x(n): its acceleration pass reuses it
        double b0 = v[0] - col(P, C_VN, N, j), b1 = v[1] - col(P, C_VN + 1, N, j), b2 = v[2] - col(P, C_VN + 2, N, j);
        {
          double dv = g.GK * (b0 * g.x0 + b1 * g.x1 + b2 * g.x2);
          bool up = nb_up(e);  // original index of j larger than i's
          // pair (P1 = smaller original index): 0.5 m_P2 (p1/d1^2 + p2/d2^2) v12.(GK x12)
          double pk = 0.5 * (up ? col(P, C_MASS, N, j) : massi) * (pri + col(P, C_PR2N, N, j)) * dv;
          dkin += up ? pk : -pk;
          if (K.thermal_solver) {
            double kj = col(P, C_KT, N, j);
            double w = up ? col(P, C_MRHON, N, j) : mrhoi;  // m_P2 / rho_P2 for both ends
            double gx[3] = {g.GK * g.x0, g.GK * g.x1, g.GK * g.x2};
            if (K.gradcorr) {  // Mult(gradCorrM_i, GK x_ij) (Thermal.cpp:90-107)
              double c3[3];
              for (int q = 0; q < 3; ++q)
                c3[q] = gx[0] * col(P, C_GCM + 3 * q, N, i) + gx[1] * col(P, C_GCM + 3 * q + 1, N, i) +
                        gx[2] * col(P, C_GCM + 3 * q + 2, N, i);
              gx[0] = c3[0]; gx[1] = c3[1]; gx[2] = c3[2];
            }
            double dxx = g.x0 * gx[0] + g.x1 * gx[1] + g.x2 * gx[2];
            cond += w * 4. * (ki * kj) / (ki + kj) * (Ti - col(P, C_TN, N, j)) * dxx / (g.r * g.r);
          }
        }
        if (K.gradcorr) {  // locking form: (float)(m_j/rho_j) with v_ij (x) vc_i (InteractionAlt.cpp:330-350, 425-450)
          double gk[3];
          corr_grad(P, N, i, g.GK, g.x0, g.x1, g.x2, gk);
          double bv[3] = {b0, b1, b2};
          double wf = (double)(float)(col(P, C_MASS, N, j) / col(P, C_RHON, N, j));
          const int ua[6] = {0, 1, 2, 0, 0, 1}, ub[6] = {0, 1, 2, 1, 2, 2};
          for (int c = 0; c < 6; ++c) {
            double gab = bv[ua[c]] * gk[ub[c]], gba = bv[ub[c]] * gk[ua[c]];
            sr[c] += wf * (-0.5 * (gab + gba));
          }
          rr[0] += wf * (-0.5 * (bv[0] * gk[1] - bv[1] * gk[0]));
          rr[1] += wf * (-0.5 * (bv[0] * gk[2] - bv[2] * gk[0]));
          rr[2] += wf * (-0.5 * (bv[1] * gk[2] - bv[2] * gk[1]));
          continue;
        }
        // (m_j/rho_j) (-GK/2) (v_ij (x) x_ij +- x_ij (x) v_ij): u = (m_j/rho_j)(-GK/2) v_ij
        // enters every entry; the diagonal collects u_a x_a and is doubled once
        // after the loop (exact in binary).
        double wf = col(P, C_MRHON, N, j) * (-0.5 * g.GK);
        double u0 = wf * b0, u1 = wf * b1, u2 = wf * b2;
        sr[0] += u0 * g.x0;
        sr[1] += u1 * g.x1;
        sr[2] += u2 * g.x2;
        sr[3] += u0 * g.x1; sr[3] += u1 * g.x0;
        sr[4] += u0 * g.x2; sr[4] += u2 * g.x0;
        sr[5] += u1 * g.x2; sr[5] += u2 * g.x1;
        rr[0] += u0 * g.x1; rr[0] -= u1 * g.x0;
        rr[1] += u0 * g.x2; rr[1] -= u2 * g.x0;
        rr[2] += u1 * g.x2; rr[2] -= u2 * g.x1;
      }
      if (!K.gradcorr)
        for (int c = 0; c < 3; ++c) sr[c] = 2.0 * sr[c];
      StressIO s;
      for (int c = 0; c < 6; ++c) {
        s.tau[c] = col(P, C_TAU + c, N, i); s.eps[c] = col(P, C_EPS + c, N, i);
        s.epl[c] = col(P, C_EPL + c, N, i); s.epli[c] = col(P, C_EPLI + c, N, i);
      }
      s.pl_strain = col(P, C_PLS, N, i); s.delta_pl_strain = col(P, C_DPLS, N, i);
      s.sigmay = col(P, C_SY, N, i); s.Ep = col(P, C_EP, N, i);
      int mi = icol(P, I_MAT, N, i);
      const MaterialDev* M = (mi >= 0 && mi < P.tab->nmat) ? &P.tab->mat[mi] : nullptr;
      double T = col(P, C_T, N, i);
      double dep = stress_update(s, sr, rr, rho, col(P, C_RHO0, N, i), col(P, C_CS, N, i), col(P, C_P0, N, i),
                                 col(P, C_G, N, i), T, icol(P, I_FAIL, N, i), icol(P, I_MODEL, N, i), M, dt);
      if (P.tx) {
        for (int c = 0; c < 6; ++c) P.tx[(size_t)(TX_SR + c) * N + i] = sr[c];
        for (int c = 0; c < 3; ++c) P.tx[(size_t)(TX_RR + c) * N + i] = rr[c];
        P.tx[(size_t)TX_SC * N + i] = s.sc;
        P.tx[(size_t)TX_SYN * N + i] = s.sy_new;
        P.tx[(size_t)TX_DEP * N + i] = dep;
      }
      for (int c = 0; c < 6; ++c) {
        colw(P, C_TAU + c, N, i) = s.tau[c]; colw(P, C_SIG + c, N, i) = s.sig[c];
        colw(P, C_EPS + c, N, i) = s.eps[c]; colw(P, C_EPL + c, N, i) = s.epl[c];
        colw(P, C_EPLI + c, N, i) = s.epli[c]; colw(P, C_SR + c, N, i) = sr[c];
      }
      for (int c = 0; c < 3; ++c) colw(P, C_RR + c, N, i) = rr[c];
      colw(P, C_P, N, i) = s.pressure; colw(P, C_PLS, N, i) = s.pl_strain; colw(P, C_DPLS, N, i) = s.delta_pl_strain;
      colw(P, C_SY, N, i) = s.sigmay; colw(P, C_EP, N, i) = s.Ep; colw(P, C_ESR, N, i) = s.esr;
      maxpl = s.pl_strain;
      mark_yield(P, K, N, i, s.pl_strain);
      double c2 = 1.0 / (rho * rho);
      for (int c = 0; c < 6; ++c) colw(P, C_SRHO + c, N, i) = c2 * s.sig[c];
      colw(P, C_PR2, N, i) = s.pressure / (rho * rho);
      double qpl = col(P, C_QPL, N, i);
      if (K.pl_heating) {
        if (s.delta_pl_strain > 0.0) qpl = plastic_heat(s.sig, s.epli, dt);
        colw(P, C_QPL, N, i) = qpl;
        colw(P, C_PSEN, N, i) = col(P, C_PSEN, N, i) + qpl * dt;
        plw = col(P, C_MASS, N, i) / rho * qpl;
      }
      double sre[6];
      for (int c = 0; c < 6; ++c) sre[c] = sr[c];
      if (K.thermal_solver) {
        T += dt * col(P, C_DTDT, N, i);
        colw(P, C_T, N, i) = T;
        maxT = T; minT = T;
        // CalcTempInc's dTdt and CalcThermalExpStrainRate (after the stress)
        double f = 1. / (rho * col(P, C_CPT, N, i));
        double qconv = conv_heat(P, N, i, rho, T);
        double dTdt = f * (cond + qconv + col(P, C_QSRC, N, i) + qpl * K.pl_work_heat_frac + 0.0);
        colw(P, C_DTDT, N, i) = dTdt;
        double st = col(P, C_THEXP, N, i) * dTdt;
        for (int c = 0; c < 3; ++c) { sre[c] = sre[c] + st; colw(P, C_SR + c, N, i) = sre[c]; }
      }
      // CalcIntEnergyEqn (Particle.cpp:941-950)
      dint = mrhoi * (s.tau[0] * sre[0] + 2.0 * s.tau[3] * sre[3] + 2.0 * s.tau[4] * sre[4] + s.tau[1] * sre[1] +
                      2.0 * s.tau[5] * sre[5] + s.tau[2] * sre[2]);
      colw(P, C_DKIN, N, i) = dkin;
      colw(P, C_DINT, N, i) = dint;
      dkin_b = dkin;
    }
  }
  double r;
  r = block_reduce<0>(dkin_b, sh); if (threadIdx.x == 0) P.partials[S_DKIN * K.nblocks + blockIdx.x] = r;
  r = block_reduce<0>(dint, sh); if (threadIdx.x == 0) P.partials[S_DINT * K.nblocks + blockIdx.x] = r;
  r = block_reduce<1>(maxpl, sh); if (threadIdx.x == 0) P.partials[S_MAXPL * K.nblocks + blockIdx.x] = r;
  if (K.pl_heating) { r = block_reduce<0>(plw, sh); if (threadIdx.x == 0) P.partials[S_PLW * K.nblocks + blockIdx.x] = r; }
  if (K.thermal_solver) {
    r = block_reduce<1>(maxT, sh); if (threadIdx.x == 0) P.partials[S_MAXT * K.nblocks + blockIdx.x] = r;
    r = block_reduce<2>(minT, sh); if (threadIdx.x == 0) P.partials[S_MINT * K.nblocks + blockIdx.x] = r;
  }
}


// ---------------------------------------------------------------- reductions
// One block per slot; each thread sums a fixed strided subset, then a fixed tree.
__global__ void k_finalize(DevPtrs P, DomainConst K) {
  __shared__ double sh[1024];
  int slot = blockIdx.x;
  bool active = (slot == S_DINT || slot == S_DKIN || slot == S_MAXPL) ||
                (K.pl_heating && slot == S_PLW) || (K.thermal_solver && (slot == S_MAXT || slot == S_MINT)) ||
                (K.contact && (slot == S_CFSUM || slot == S_CRSUM || slot == S_EXTW ||
                               (slot >= S_CFVEC && slot < S_CFVEC + 3 * K.nmeshes)));
  if (!active) return;
  int op = (slot == S_MAXPL || slot == S_MAXT) ? 1 : (slot == S_MINT ? 2 : 0);
  double acc = op == 1 ? -1e300 : (op == 2 ? 1e300 : 0.0);
  const double* src = P.partials + (size_t)slot * K.nblocks;
  for (int b = threadIdx.x; b < K.nblocks; b += blockDim.x) {
    double v = src[b];
    acc = op == 0 ? acc + v : (op == 1 ? fmax(acc, v) : fmin(acc, v));
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      double a = sh[threadIdx.x], b = sh[threadIdx.x + s];
      sh[threadIdx.x] = op == 0 ? a + b : (op == 1 ? fmax(a, b) : fmin(a, b));
    }
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  double v = sh[0];
  StepState* st = P.st;
  double dt = st->deltat;
  switch (slot) {
    case S_DINT:
      st->int_energy_sum += v * dt;
      if (K.nan_check && !isfinite(v)) atomicOr(&st->errors, ERR_NAN);
      break;
    case S_DKIN:
      st->kin_energy_sum += v * dt;
      if (K.nan_check && !isfinite(v)) atomicOr(&st->errors, ERR_NAN);
      break;
    case S_PLW: st->plastic_work += v * dt; break;
    case S_MAXPL: st->max_pl_next = v; break;
    case S_MAXT: st->m_maxT = v > 0.0 ? v : 0.0; break;
    case S_MINT: st->m_minT = v < 1000. ? v : 1000.; break;
    case S_CFSUM: st->contact_force_sum = v; break;
    case S_CRSUM: st->contact_reaction_sum = v; break;
    case S_EXTW: st->ext_forces_work += v * dt; break;
    default: {
      int q = slot - S_CFVEC;
      st->contact_force[q / 3][q % 3] = v;
    }
  }
}

// ---------------------------------------------------------------- rigid meshes
// TriMesh::Update: node_v = m_v + m_w x node; node += node_v dt.
__global__ void k_mesh_nodes(DevPtrs P, DomainConst K) {
  int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= P.nnodes) return;
  int m = P.node_mesh[n];
  const double* mv = P.st->mesh_v[m];
  const double* mw = P.st->mesh_w[m];
  double p[3] = {P.node[n], P.node[P.nnodes + n], P.node[2 * P.nnodes + n]};
  double vr[3] = {mw[1] * p[2] - mw[2] * p[1], mw[2] * p[0] - mw[0] * p[2], mw[0] * p[1] - mw[1] * p[0]};
  if (!K.contact_mesh_auto_update) return;
  for (int d = 0; d < 3; ++d) {
    double nv = mv[d] + vr[d];
    P.node_v[d * P.nnodes + n] = nv;
    P.node[d * P.nnodes + n] = p[d] + nv * P.st->deltat;
  }
}
// CalcNormals + UpdatePlaneCoeff per element (Mesh.cpp:222-256), then
// UpdateContactParticles (Contact.cpp:41-55) for the element's particle.
__global__ void k_mesh_elems(DevPtrs P, DomainConst K) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= P.nelem) return;
  int nn = P.nnodes;
  int n0 = P.elem_node[3 * e], n1 = P.elem_node[3 * e + 1], n2 = P.elem_node[3 * e + 2];
  size_t N = K.N;
  int p = P.elem_particle[e];
  double nrm[3] = {P.elem_normal[e], P.elem_normal[P.nelem + e], P.elem_normal[2 * P.nelem + e]};
  if (K.contact_mesh_auto_update) {
    double a[3] = {P.node[n0], P.node[nn + n0], P.node[2 * nn + n0]};
    double b[3] = {P.node[n1], P.node[nn + n1], P.node[2 * nn + n1]};
    double c[3] = {P.node[n2], P.node[nn + n2], P.node[2 * nn + n2]};
    double u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, w[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    double cr[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
    double ln = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    for (int d = 0; d < 3; ++d) { nrm[d] = cr[d] / ln; P.elem_normal[d * P.nelem + e] = nrm[d]; }
    P.elem_pplane[e] = c[0] * nrm[0] + c[1] * nrm[1] + c[2] * nrm[2];  // nfar = last node
  }
  for (int d = 0; d < 3; ++d) {
    double s = 0.0;
    s = s + P.node_v[d * nn + n0]; s = s + P.node_v[d * nn + n1]; s = s + P.node_v[d * nn + n2];
    colw(P, C_V + d, N, p) = s / 3;
    colw(P, C_A + d, N, p) = 0.0;
    colw(P, C_NORMAL + d, N, p) = nrm[d];
    if (K.mixed) rec_set_v(P, N, p, d, s / 3, false);
  }
}

// ---------------------------------------------------------------- prologue helpers
__global__ void k_refresh_derived(DevPtrs P, DomainConst K) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K.N) return;
  size_t N = K.N;
  if (icol(P, I_KIND, N, i) != 0) {  // rigid-mesh particles carry no mass or density
    for (int c = 0; c < 6; ++c) colw(P, C_SRHO + c, N, i) = 0.0;
    colw(P, C_MRHO, N, i) = 0.0;
    colw(P, C_PR2, N, i) = 0.0;
    return;
  }
  double rho = col(P, C_RHO, N, i);
  double c2 = 1.0 / (rho * rho);
  for (int c = 0; c < 6; ++c) colw(P, C_SRHO + c, N, i) = c2 * col(P, C_SIG + c, N, i);
  colw(P, C_MRHO, N, i) = col(P, C_MASS, N, i) / rho;
  colw(P, C_PR2, N, i) = col(P, C_P, N, i) / (rho * rho);
}
__global__ void k_initial_pressure(DevPtrs P, DomainConst K) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K.N) return;
  size_t N = K.N;
  double cs = col(P, C_CS, N, i);
  colw(P, C_P, N, i) = col(P, C_P0, N, i) + (cs * cs) * (col(P, C_RHO, N, i) - col(P, C_RHO0, N, i));
}
__global__ void k_max_pl(DevPtrs P, DomainConst K) {
  __shared__ double sh[32];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double v = (i < K.N) ? col(P, C_PLS, (size_t)K.N, i) : 0.0;
  double r = block_reduce<1>(v, sh);
  if (threadIdx.x == 0) P.partials[S_MAXPL * K.nblocks + blockIdx.x] = r;
}
__global__ void k_max_pl_final(DevPtrs P, DomainConst K) {
  if (threadIdx.x || blockIdx.x) return;
  double m = 0.0;
  for (int b = 0; b < K.nblocks; ++b) m = fmax(m, P.partials[S_MAXPL * K.nblocks + b]);
  P.st->max_pl_next = m;
}

void launch_prologue(const DevPtrs& P, const DomainConst& K, cudaStream_t s) {
  k_initial_pressure<<<nblk(K.N, BLOCK), BLOCK, 0, s>>>(P, K);
  k_refresh_derived<<<nblk(K.N, BLOCK), BLOCK, 0, s>>>(P, K);
  k_max_pl<<<K.nblocks, K.pblock, 0, s>>>(P, K);
  k_max_pl_final<<<1, 1, 0, s>>>(P, K);
}
void launch_refresh_derived(const DevPtrs& P, const DomainConst& K, cudaStream_t s) {
  k_refresh_derived<<<nblk(K.N, BLOCK), BLOCK, 0, s>>>(P, K);
}

// ---------------------------------------------------------------- host transfers
__global__ void k_gather_orig(DevPtrs P, DomainConst K, const double* colp, double* out, int ncomp) {
  int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= K.N) return;
  int i = P.inv[o];
  for (int c = 0; c < ncomp; ++c) out[(size_t)o * ncomp + c] = colp[(size_t)c * K.N + i];
}
__global__ void k_scatter_orig(DevPtrs P, DomainConst K, const double* in, double* colp, int ncomp) {
  int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= K.N) return;
  int i = P.inv[o];
  for (int c = 0; c < ncomp; ++c) colp[(size_t)c * K.N + i] = in[(size_t)o * ncomp + c];
}
// A stored symmetric tensor (xx, yy, zz, xy, xz, yz) or antisymmetric one
// (xy, xz, yz) written as full row-major 3x3 rows in original order.
__global__ void k_gather_orig_tensor(DevPtrs P, DomainConst K, const double* colp, double* out, int anti) {
  int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= K.N) return;
  const size_t N = K.N;
  int i = P.inv[o];
  double* r = out + (size_t)o * 9;
  if (anti) {
    double a = colp[i], b = colp[N + i], c = colp[2 * N + i];
    r[0] = 0.0; r[1] = a; r[2] = b;
    r[3] = -a; r[4] = 0.0; r[5] = c;
    r[6] = -b; r[7] = -c; r[8] = 0.0;
  } else {
    double xx = colp[i], yy = colp[N + i], zz = colp[2 * N + i];
    double xy = colp[3 * N + i], xz = colp[4 * N + i], yz = colp[5 * N + i];
    r[0] = xx; r[1] = xy; r[2] = xz;
    r[3] = xy; r[4] = yy; r[5] = yz;
    r[6] = xz; r[7] = yz; r[8] = zz;
  }
}
__global__ void k_gather_orig_i32(DevPtrs P, DomainConst K, const int* colp, int* out) {
  int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= K.N) return;
  out[o] = colp[P.inv[o]];
}
__global__ void k_scatter_orig_i32(DevPtrs P, DomainConst K, const int* in, int* colp) {
  int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= K.N) return;
  colp[P.inv[o]] = in[o];
}
void launch_gather_orig(const DevPtrs& P, const DomainConst& K, const double* c, double* o, int n, cudaStream_t s) {
  k_gather_orig<<<nblk(K.N, BLOCK), BLOCK, 0, s>>>(P, K, c, o, n);
}
void launch_scatter_orig(const DevPtrs& P, const DomainConst& K, const double* in, double* c, int n, cudaStream_t s) {
  k_scatter_orig<<<nblk(K.N, BLOCK), BLOCK, 0, s>>>(P, K, in, c, n);
}
void launch_gather_orig_tensor(const DevPtrs& P, const DomainConst& K, const double* c, double* o, int anti,
                               cudaStream_t s) {
  k_gather_orig_tensor<<<nblk(K.N, BLOCK), BLOCK, 0, s>>>(P, K, c, o, anti);
}
void launch_gather_orig_i32(const DevPtrs& P, const DomainConst& K, const int* c, int* o, cudaStream_t s) {
  k_gather_orig_i32<<<nblk(K.N, BLOCK), BLOCK, 0, s>>>(P, K, c, o);
}
void launch_scatter_orig_i32(const DevPtrs& P, const DomainConst& K, const int* in, int* c, cudaStream_t s) {
  k_scatter_orig_i32<<<nblk(K.N, BLOCK), BLOCK, 0, s>>>(P, K, in, c);
}

// ---------------------------------------------------------------- one step
void launch_step_head(const DevPtrs& P, const DomainConst& K, double* fscratch, int* iscratch, cudaStream_t s) {
  SearchCond* c = g_search_cond;
  unsigned long long cond = c ? c->begin(s) : 0ull;
  k_schedule<<<1, 256, 0, s>>>(P, K, cond);
  mark(s, "k_schedule");
  cudaStream_t ss = c ? c->open_body(s) : s;
  launch_neighbour_search(P, K, fscratch, iscratch, ss);
  if (K.mixed) launch_refresh_shadows(P, K, 0, ss);  // after a search that reordered the particles
  if (c) c->close_body();
  if (K.gradcorr) {
    int b = K.nblocks;
    k_grad_corr<<<b < 152 * 8 ? b : 152 * 8, K.pblock, 0, s>>>(P, K);
    mark(s, "k_grad_corr");
  }
}
// ---------------------------------------------------------------- adaptive time step
// CheckMinTSVel (Domain.cpp:265-299): CFL * (shortest neighbour distance, 1000
// without neighbours) / (Cs + |v|); CheckMinTSAccel (:304-319):
// sqrt_h_a * sqrt(h / |a|).  Every particle; block minima into S_DTV / S_DTA.
__global__ void __launch_bounds__(BLOCK) k_dt_tests(DevPtrs P, DomainConst K, int vel, int acc) {
  __shared__ double sh[32];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  size_t N = K.N;
  double tv = 1.0 / 0.0, ta = 1.0 / 0.0;
  if (i < K.N) {
    if (vel) {
      double xi[3] = {col(P, C_X, N, i), col(P, C_X + 1, N, i), col(P, C_X + 2, N, i)};
      double mn = 1000.;
      int len = P.row_len[i];
      for (int k = 0; k < len; ++k) {
        int j = nb_index(P.nbr[(size_t)k * N + i]);
        double d0 = col(P, C_X, N, j) - xi[0], d1 = col(P, C_X + 1, N, j) - xi[1], d2 = col(P, C_X + 2, N, j) - xi[2];
        double d = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
        if (d < mn) mn = d;
      }
      double v0 = col(P, C_V, N, i), v1 = col(P, C_V + 1, N, i), v2 = col(P, C_V + 2, N, i);
      tv = K.CFL * mn / (col(P, C_CS, N, i) + sqrt(v0 * v0 + v1 * v1 + v2 * v2));
    }
    if (acc) {
      double a0 = col(P, C_A, N, i), a1 = col(P, C_A + 1, N, i), a2 = col(P, C_A + 2, N, i);
      ta = K.sqrt_h_a * sqrt(col(P, C_H, N, i) / sqrt(a0 * a0 + a1 * a1 + a2 * a2));
    }
  }
  double r;
  if (vel) { r = block_reduce<2>(tv, sh); if (threadIdx.x == 0) P.partials[S_DTV * K.nblocks + blockIdx.x] = r; }
  if (acc) { r = block_reduce<2>(ta, sh); if (threadIdx.x == 0) P.partials[S_DTA * K.nblocks + blockIdx.x] = r; }
}

// AdaptiveTimeStep (Domain.cpp:206-239) from the candidates' minimum.  Each
// criterion starts from deltatint and the acceleration one runs second, so
// with both on only it counts (CheckMinTSAccel resets deltatmin).  The
// contact term cannot lower deltat here (the leapfrog solver's min_force_ts
// is the initial dt; kick-drift with it is rejected) and the floor
// manual_min_ts is an int member holding 0 (Domain.h:328).
__global__ void k_adapt_dt(DevPtrs P, DomainConst K) {
  __shared__ double sh[32];
  double mv = 1.0 / 0.0, ma = 1.0 / 0.0;
  for (int b = threadIdx.x; b < K.nblocks; b += blockDim.x) {
    if (K.auto_ts) mv = fmin(mv, P.partials[S_DTV * K.nblocks + b]);
    if (K.auto_ts_acc) ma = fmin(ma, P.partials[S_DTA * K.nblocks + b]);
  }
  mv = block_reduce<2>(mv, sh);
  ma = block_reduce<2>(ma, sh);
  if (threadIdx.x != 0) return;
  StepState* st = P.st;
  double dint = st->deltatint, dmin = dint;
  if (K.auto_ts) dmin = fmin(dint, mv);
  if (K.auto_ts_acc) dmin = fmin(dint, ma);
  double dt = st->deltat;
  st->prev_deltat = dt;
  if (dint > dmin) dt = dt < dmin ? 2.0 * dt * dmin / (dt + dmin) : dmin;
  else dt = dint != dt ? 2.0 * dt * dint / (dt + dint) : dint;
  st->deltat = dt;
}

void launch_bc(const DevPtrs& P, const DomainConst& K, int vcol, cudaStream_t s) {
  int nbc = nblk(K.nbc_particles > 0 ? K.nbc_particles : 1, BLOCK);
  k_bc<<<nbc, BLOCK, 0, s>>>(P, K, vcol);
  mark(s, "k_bc");
}
void launch_contact_kick(const DevPtrs& P, const DomainConst& K, cudaStream_t s) {
  bool adapt = K.auto_ts || K.auto_ts_acc;
  if (K.auto_ts && !K.leapfrog) {  // kick-drift: the velocity criterion sees v before the first kick
    k_dt_tests<<<K.nblocks, K.pblock, 0, s>>>(P, K, 1, 0);
    mark(s, "k_dt_tests");
  }
  if (!K.contact) k_contact_kick<0><<<K.nblocks, K.pblock, 0, s>>>(P, K);
  else if (K.nmeshes == 1) k_contact_kick<1><<<K.nblocks, K.pblock, 0, s>>>(P, K);
  else k_contact_kick<MAX_MESHES><<<K.nblocks, K.pblock, 0, s>>>(P, K);
  mark(s, "k_contact_kick");
  if (K.leapfrog) {  // GeneralAfter, time-step control, then the full kick (the caller's BC pass follows)
    launch_bc(P, K, C_V, s);
    if (adapt) {
      k_dt_tests<<<K.nblocks, K.pblock, 0, s>>>(P, K, K.auto_ts, K.auto_ts_acc);
      mark(s, "k_dt_tests");
      k_adapt_dt<<<1, 256, 0, s>>>(P, K);
      mark(s, "k_adapt_dt");
    }
    k_kick_leapfrog<<<K.nblocks, K.pblock, 0, s>>>(P, K);
    mark(s, "k_kick_leapfrog");
  } else if (adapt) {
    k_adapt_dt<<<1, 256, 0, s>>>(P, K);
    mark(s, "k_adapt_dt");
  }
}
void launch_step_tail(const DevPtrs& P, const DomainConst& K, cudaStream_t s) {
  k_finalize<<<NSLOTS, 1024, 0, s>>>(P, K);
  mark(s, "k_finalize");
  if (K.contact && P.nelem > 0) {
    k_mesh_nodes<<<nblk(P.nnodes, BLOCK), BLOCK, 0, s>>>(P, K);
    mark(s, "k_mesh_nodes");
    k_mesh_elems<<<nblk(P.nelem, BLOCK), BLOCK, 0, s>>>(P, K);
    mark(s, "k_mesh_elems");
  }
  k_step_end<<<1, 256, 0, s>>>(P, K);
  mark(s, "k_step_end");
}

void launch_step_fp64(const DevPtrs& P, const DomainConst& K, double* fscratch, int* iscratch, cudaStream_t s) {
  launch_step_head(P, K, fscratch, iscratch, s);
  launch_step_fp64_body(P, K, s);
}

void launch_tensile(const DevPtrs& P, const DomainConst& K, cudaStream_t s) {
  if (!K.ti) return;
  k_tensile<<<K.nblocks, K.pblock, 0, s>>>(P, K);
  mark(s, "k_tensile");
}

void launch_step_fp64_body(const DevPtrs& P, const DomainConst& K, cudaStream_t s) {
  int nb = K.nblocks;
  launch_tensile(P, K, s);
  k_accel<<<nb, K.pblock, 0, s>>>(P, K);
  mark(s, "k_accel");
  launch_bc(P, K, C_V, s);
  launch_contact_kick(P, K, s);
  if (K.leapfrog) launch_bc(P, K, C_V, s);  // kick-drift: applied by the kick kernel
  k_density_drift<<<nb, K.pblock, 0, s>>>(P, K);  // and the next-step BC by this one
  mark(s, "k_density_drift");
  k_rate_stress<<<nb, K.pblock, 0, s>>>(P, K);
  mark(s, "k_rate_stress");
  launch_step_tail(P, K, s);
}

}  // namespace wf
