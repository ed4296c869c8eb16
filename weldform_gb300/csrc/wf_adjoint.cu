// Reverse-mode kernels of one plain FP64 kick-drift step.
//
// Forward step (Domain::SolveDiffUpdateKickDrift, SolverKickDrift.cpp:117-393),
// written as the maps the reverse pass inverts, for solid particle i:
//   A  a0   = sum_j +-m_j PF(x, v, rho, Sigma, Cs)       CalcAccel (InteractionAlt.cpp:12-260)
//   B1 BC particles: a0 = 0, v1 = v_bc                    GeneralAfter (WeldForm.cpp:51-120)
//   C  a1   = a0 + contact(x, v1, a0, rho) / m            CalcContactForcesWang (Contact_Wang.cpp:15-348)
//   D  vh   = v1 + a1 dt/2;  B2: BC -> vh = v_bc, a2 = 0
//   F  rho' = rho + dt rho sum_j (m_j/rho_j) vh_ij.GK x_ij CalcDensInc (InteractionAlt.cpp:483-640)
//   G  x'   = x + dt vh;  H  v' = vh + a2 dt/2;  B3: BC -> v' = v_bc
//   J  SR, RR = sum_j (m_j/rho'_j) rates(x', v')          CalcRateTensors (InteractionAlt.cpp:263-479)
//   K  radial return -> tau', Sigma', pl', Sigmay', Inc'  CalcStressStrain (Particle.cpp:960-1067)
//   L  q_pl = Sigma':Inc'/dt once yielded                 CalcPlasticWorkHeat (Particle.cpp:922-939)
//   M  T' = T + dt dTdt;  dTdt' = (cond(x', rho', T') + q_src + frac q_pl) / (rho' cp)
//                                                          ThermalCalcs (Thermal.cpp:721-748)
// Energies and the rigid-mesh update feed nothing back and have no adjoint.
//
// Four kernels, each one thread per particle (gathers over the particle's own
// neighbour row, so every adjoint sum is a deterministic per-particle sum):
//   R1 M + K + L   thermal gather (end state) and the radial-return adjoint
//   R2 J + H + G   rate gather (end state), second kick and drift
//   R3 F + D + C   density gather (start state), first kick, contact pairs
//   R4 A           acceleration gather (start state)
// A pair term f(x_i - x_j, ...) enters the sums of both ends; each end's
// thread differentiates the pair's total contribution with respect to its own
// variables, reading the partner's adjoint from the previous kernel.
#include "wf_adjoint.cuh"
#include "wf_step_common.cuh"
#include "wf_launch.h"

namespace wf {

static inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }
static_assert(ADJ_BLOCK == BLOCK, "the finish kernel's partials are sized by ADJ_BLOCK");

// Cubic-spline gradient kernel (Functions.cpp:74-87) and its derivative in r,
// with C = 1 / (pi hh^4):
//   q < 1:      GK = C/hh (-3 + 9/4 q),     dGK/dr = C/hh^2 9/4
//   1 <= q < 2: GK = -3/4 C (2 - q)^2 / r,  dGK/dr = 3/4 C (4 - q^2) / r^2
// with r and 1/r from one reciprocal square root per pair, plus 1/hh when
// the pair's smoothing lengths differ (inv_hi = 1/h_i is the caller's).  The
// values equal the forward's to rounding.
struct GeoD {
  double x0, x1, x2, r, GK, dGr;  // dGr = (dGK/dr) / r
};
__device__ __forceinline__ GeoD geo_d(const double xi[3], double hi, double inv_hi, double xj0, double xj1, double xj2,
                                      double hj) {
  GeoD g;
  g.x0 = xi[0] - xj0; g.x1 = xi[1] - xj1; g.x2 = xi[2] - xj2;
  double r2 = g.x0 * g.x0 + g.x1 * g.x1 + g.x2 * g.x2;
  double rinv = r2 > 0.0 ? rsqrt(r2) : 0.0;
  g.r = r2 * rinv;
  double inv_h = hj == hi ? inv_hi : 2.0 / (hi + hj);
  double q = g.r * inv_h;
  double ih2 = inv_h * inv_h;
  double C = ih2 * ih2 * (1.0 / WF_PI);
  double dG = 0.0;
  if (q == 0.0) g.GK = C * inv_h * -3.0;
  else if (q < 1.0) { g.GK = C * inv_h * (-3.0 + 2.25 * q); dG = C * ih2 * 2.25; }
  else if (q < 2.0) {
    double t = 2.0 - q;
    g.GK = C * rinv * (-0.75 * t * t);
    dG = C * 0.75 * (4.0 - q * q) * (rinv * rinv);
  } else g.GK = 0.0;
  g.dGr = dG * rinv;
  return g;
}

// Velocity BC of a zone at time t (GeneralAfter): true if a BC applies, with
// its value in vb (the last matching BC wins, as the forward loop).
__device__ __forceinline__ bool bc_value(const DomainTables* T, int id, double t, double vb[3]) {
  bool hit = false;
  int lo, hi;
  bc_range(T, id, lo, hi);
  for (int r = lo; r < hi; ++r) {
    const int b = T->bc_order[r];
    if (T->bc[b].value_type == 0) {
      hit = true;
      for (int d = 0; d < 3; ++d) vb[d] = T->bc[b].value[d];
    } else {
      bool found = false;
      double val = T->bc[b].amp_factor * amp_value(T, T->bc[b].amp_id, t, &found);
      if (found) {
        hit = true;
        for (int d = 0; d < 3; ++d) vb[d] = val * T->bc[b].value[d];
      }
    }
  }
  return hit;
}

#define FE(c, p) A.fe[(size_t)(c) * N + (p)]
#define TXV(c, p) A.tx[(size_t)(c) * N + (p)]
#define LIN(c, p) A.Lin[(size_t)(c) * N + (p)]
#define LOUT(c) A.Lout[(size_t)(c) * N + i]
#define TMP(c, p) A.Tmp[(size_t)(c) * N + (p)]
#define QA(c) A.Q[(size_t)(c) * N + i]

// ---------------------------------------------------------------- R1: thermal + radial return
__global__ void __launch_bounds__(BLOCK) k_adj_thermal_stress(AdjPtrs A, DomainConst K) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K.N) return;
  const DevPtrs& S = A.S;
  size_t N = K.N;
  double dt = K.dt;
  if (icol(S, I_KIND, N, i) != 0) {
    for (int c = 0; c < 6; ++c) { LOUT(A_TAU + c) = 0.0; LOUT(A_INC + c) = 0.0; TMP(J_SR + c, i) = 0.0; }
    for (int c = 0; c < 3; ++c) { TMP(J_RR + c, i) = 0.0; TMP(J_XN + c, i) = 0.0; TMP(J_VN + c, i) = 0.0; }
    LOUT(A_PLS) = 0.0; LOUT(A_SY) = 0.0; LOUT(A_T) = 0.0; LOUT(A_DTDT) = 0.0; TMP(J_RHON, i) = 0.0;
    return;
  }
  double lxn[3] = {LIN(A_X, i), LIN(A_X + 1, i), LIN(A_X + 2, i)};
  double lrhon = LIN(A_RHO, i);
  double ltn = LIN(A_T, i);
  double rhoN = FE(C_RHO, i);
  double lqpl = 0.0;
  // ---- M: T' = T + dt dTdt, dTdt' = (cond + q_src + frac q_pl) / (rho' cp)
  if (K.thermal_solver) {
    double ldT = LIN(A_DTDT, i);
    double lci = TMP(J_LC, i);
    double inv_rhoN = 1.0 / rhoN;
    lrhon += -FE(C_DTDT, i) * ldT * inv_rhoN;
    if (K.pl_heating) lqpl = K.pl_work_heat_frac * lci;
    double xi[3] = {FE(C_X, i), FE(C_X + 1, i), FE(C_X + 2, i)};
    double hi = col(S, C_H, N, i), ki = col(S, C_KT, N, i), Ti = FE(C_T, i), wi = FE(C_MRHO, i);
    double inv_hi = 1.0 / hi;
    int len = S.row_len[i];
    for (int k = 0; k < len; ++k) {
      int e = S.nbr[(size_t)k * N + i];
      int j = nb_index(e);
      GeoD g = geo_d(xi, hi, inv_hi, FE(C_X, j), FE(C_X + 1, j), FE(C_X + 2, j), col(S, C_H, N, j));
      A.gk_end[(size_t)k * N + i] = g.GK;  // R2 reads the same end-state geometry
      A.dg_end[(size_t)k * N + i] = g.dGr;
      double lcj = TMP(J_LC, j);
      double d = lci - lcj;
      bool up = nb_up(e);  // j has the larger original index: P2 = j
      double w = up ? FE(C_MRHO, j) : wi;  // m_P2 / rho_P2 at both ends (Thermal.cpp:127-131)
      double kj = col(S, C_KT, N, j);
      double kk = 4. * (ki * kj) / (ki + kj);
      double dT = Ti - FE(C_T, j);
      ltn += d * w * kk * g.GK;
      double cx = d * w * kk * dT * g.dGr;
      lxn[0] += cx * g.x0; lxn[1] += cx * g.x1; lxn[2] += cx * g.x2;
      if (!up) lrhon += -d * w * kk * dT * g.GK * inv_rhoN;
    }
  }
  // ---- K + L: radial return (Particle.cpp:960-1067) and plastic-work heat
  double tau[6], sr[6], rr[3];
  for (int c = 0; c < 6; ++c) { tau[c] = col(S, C_TAU + c, N, i); sr[c] = TXV(TX_SR + c, i); }
  for (int c = 0; c < 3; ++c) rr[c] = TXV(TX_RR + c, i);
  double G = col(S, C_G, N, i), Cs = col(S, C_CS, N, i), rho0 = col(S, C_RHO0, N, i), Ep = col(S, C_EP, N, i);
  double Sm[3][3] = {{tau[0], tau[3], tau[4]}, {tau[3], tau[1], tau[5]}, {tau[4], tau[5], tau[2]}};
  double W[3][3] = {{0.0, rr[0], rr[1]}, {-rr[0], 0.0, rr[2]}, {-rr[1], -rr[2], 0.0}};
  const int ui[6] = {0, 1, 2, 0, 0, 1}, uj[6] = {0, 1, 2, 1, 2, 2};
  double s3 = 1.0 / 3.0 * (sr[0] + sr[1] + sr[2]);
  double twoG = 2.0 * G;
  double t6[6], dev[6];
  for (int c = 0; c < 6; ++c) {
    int a = ui[c], b = uj[c];
    double srt = Sm[a][2] * W[b][2] + Sm[a][1] * W[b][1] + Sm[a][0] * W[b][0];
    double rs = W[a][2] * Sm[2][b] + W[a][1] * Sm[1][b] + W[a][0] * Sm[0][b];
    dev[c] = sr[c] - (c < 3 ? s3 : 0.0);
    t6[c] = dt * (twoG * dev[c] + srt + rs) + tau[c];
  }
  int fail = icol(S, I_FAIL, N, i), model = icol(S, I_MODEL, N, i), mi = icol(S, I_MAT, N, i);
  const MaterialDev* M = (mi >= 0 && mi < S.tab->nmat) ? &S.tab->mat[mi] : nullptr;
  double sc = TXV(TX_SC, i), dep = TXV(TX_DEP, i);
  double pls0 = col(S, C_PLS, N, i), T0 = col(S, C_T, N, i);
  double syE = FE(C_SY, i), esr = FE(C_ESR, i);
  double sigE[6], incE[6], lsig[6], ltau[6], linc[6];
  for (int c = 0; c < 6; ++c) {
    sigE[c] = FE(C_SIG + c, i); incE[c] = FE(C_EPLI + c, i);
    lsig[c] = LIN(A_SIG + c, i); ltau[c] = LIN(A_TAU + c, i); linc[c] = LIN(A_INC + c, i);
  }
  double lpls = LIN(A_PLS, i), lsy = LIN(A_SY, i);
  // L: q_pl = Sigma':Inc'/dt (off-diagonal pairs doubled) while delta_pl_strain > 0
  if (lqpl != 0.0 && FE(C_DPLS, i) > 0.0) {
    double f = 1. / dt;
    for (int c = 0; c < 6; ++c) {
      double wc = c < 3 ? 1.0 : 2.0;
      lsig[c] += lqpl * wc * (f * incE[c]);
      linc[c] += lqpl * wc * f * sigE[c];
    }
  }
  bool yielded = fail == 1 && dep > 0.0;
  double ldep = 0.0, lsytot = lsy;
  double linc0[6];
  if (yielded) {  // Inc' = (dep / Sigmay') D(Sigma')
    double D[6] = {sigE[0] - 0.5 * (sigE[1] + sigE[2]), sigE[1] - 0.5 * (sigE[0] + sigE[2]),
                   sigE[2] - 0.5 * (sigE[0] + sigE[1]), 1.5 * sigE[3], 1.5 * sigE[4], 1.5 * sigE[5]};
    double f = dep / syE;
    double lf = 0.0, lD[6];
    for (int c = 0; c < 6; ++c) { lf += linc[c] * D[c]; lD[c] = f * linc[c]; }
    lsig[0] += lD[0] - 0.5 * lD[1] - 0.5 * lD[2];
    lsig[1] += lD[1] - 0.5 * lD[0] - 0.5 * lD[2];
    lsig[2] += lD[2] - 0.5 * lD[0] - 0.5 * lD[1];
    for (int c = 3; c < 6; ++c) lsig[c] += 1.5 * lD[c];
    ldep += lf / syE;
    lsytot -= lf * dep / (syE * syE);
    for (int c = 0; c < 6; ++c) linc0[c] = 0.0;
  } else {
    for (int c = 0; c < 6; ++c) linc0[c] = linc[c];
  }
  // Sigma' = -p' I + tau', p' = P0 + Cs^2 (rho' - rho0)
  double lts[6];
  for (int c = 0; c < 6; ++c) lts[c] = ltau[c] + lsig[c];
  double lp = -(lsig[0] + lsig[1] + lsig[2]);
  lrhon += lp * (Cs * Cs);
  double lCs = lp * 2.0 * Cs * (rhoN - rho0);
  double lG = 0.0, lEp = 0.0, lpls0 = lpls, lsy0 = 0.0, lT0 = 0.0, lesr = 0.0;
  double lt6[6];
  if (fail == 1) {
    double J2 = 0.5 * (t6[0] * t6[0] + 2.0 * t6[3] * t6[3] + 2.0 * t6[4] * t6[4] + t6[1] * t6[1] +
                       2.0 * t6[5] * t6[5] + t6[2] * t6[2]);
    double sigt = sqrt(3.0 * J2);
    double lsigt = 0.0, lsyn;
    if (yielded) {  // pl' = pl + dep; Sigmay' = syn (+ dep Ep, bilinear); dep = (sig_t - syn) / (3G + Ep)
      ldep += lpls;
      lsyn = lsytot;
      if (model == 0) { ldep += lsytot * Ep; lEp += lsytot * dep; }
      double den = 3. * G + Ep;
      lsigt += ldep / den;
      lsyn -= ldep / den;
      lG -= 3.0 * ldep * dep / den;
      lEp -= ldep * dep / den;
    } else {
      lsyn = lsytot;
    }
    // syn: Hollomon / Johnson-Cook flow stress, or Sigmay itself (bilinear)
    if (model == 1 && M) {
      if (pls0 + M->eps0 > M->eps1) lpls0 += lsyn * M->K * M->m * pow(pls0 + M->eps0, M->m - 1.0);
    } else if (model == 2 && M) {
      double pn = pow(pls0, M->n);
      double P1 = M->A + M->B * pn;
      bool rate = esr > M->eps_0;
      double lnr = rate ? log(esr / M->eps_0) : 0.0;
      double F = rate ? (1.0 + M->C * lnr) : 1.0;
      double Th = (T0 - M->T_t) / (M->T_m - M->T_t);
      double Thm = pow(Th, M->jm);
      double Qt = 1.0 - Thm;
      double lP1 = lsyn * F * Qt, lF = lsyn * P1 * Qt, lQ = lsyn * P1 * F;
      QA(Q_A) += lP1;
      QA(Q_B) += lP1 * pn;
      if (pls0 > 0.0) {
        lpls0 += lP1 * M->B * M->n * pow(pls0, M->n - 1.0);
        QA(Q_N) += lP1 * M->B * pn * log(pls0);
      }
      if (rate) { QA(Q_C) += lF * lnr; lesr += lF * M->C / esr; }
      double dQ = -(M->jm == 1.0 ? 1.0 : (Th > 0.0 ? M->jm * pow(Th, M->jm - 1.0) : 0.0));
      lT0 += lQ * dQ / (M->T_m - M->T_t);
      if (Th > 0.0) QA(Q_M) += -lQ * Thm * log(Th);
    } else {
      lsy0 += lsyn;
    }
    // tau_s = sc tau_trial, sc = min(Sigmay / sig_t, 1)
    double lsc = 0.0;
    for (int c = 0; c < 6; ++c) { lt6[c] = sc * lts[c]; lsc += lts[c] * t6[c]; }
    if (sc < 1.0 && sigt > 0.0) {
      lsy0 += lsc / sigt;
      lsigt -= lsc * sc / sigt;
    }
    if (sigt > 0.0) {
      double lJ2 = lsigt * 1.5 / sigt;
      for (int c = 0; c < 6; ++c) lt6[c] += lJ2 * (c < 3 ? t6[c] : 2.0 * t6[c]);
    }
  } else {
    for (int c = 0; c < 6; ++c) lt6[c] = lts[c];
    lsy0 = lsy;
  }
  // eff_strain_rate -> StrainRate
  double lsr[6] = {0, 0, 0, 0, 0, 0}, lrr[3];
  if (lesr != 0.0 && esr > 0.0) {
    double lE2 = lesr / (2.0 * esr);
    double d01 = sr[0] - sr[1], d12 = sr[1] - sr[2], d20 = sr[2] - sr[0];
    lsr[0] += lE2 * (d01 - d20); lsr[1] += lE2 * (d12 - d01); lsr[2] += lE2 * (d20 - d12);
    lsr[3] += lE2 * 6.0 * sr[3]; lsr[4] += lE2 * 6.0 * sr[4]; lsr[5] += lE2 * 6.0 * sr[5];
  }
  // tau_trial = dt (2G dev(SR) + tau W^T + W tau) + tau
  double ltau0[6], lS[3][3], lW[3][3];
  for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) { lS[a][b] = 0.0; lW[a][b] = 0.0; }
  double ls3 = 0.0;
  for (int c = 0; c < 6; ++c) {
    ltau0[c] = lt6[c];
    int a = ui[c], b = uj[c];
    double l = dt * lt6[c];
    lG += 2.0 * l * dev[c];
    double ldev = l * twoG;
    lsr[c] += ldev;
    if (c < 3) ls3 -= ldev;
    for (int k = 0; k < 3; ++k) {
      lS[a][k] += l * W[b][k]; lW[b][k] += l * Sm[a][k];
      lW[a][k] += l * Sm[k][b]; lS[k][b] += l * W[a][k];
    }
  }
  for (int c = 0; c < 3; ++c) lsr[c] += ls3 / 3.0;
  ltau0[0] += lS[0][0]; ltau0[1] += lS[1][1]; ltau0[2] += lS[2][2];
  ltau0[3] += lS[0][1] + lS[1][0]; ltau0[4] += lS[0][2] + lS[2][0]; ltau0[5] += lS[1][2] + lS[2][1];
  lrr[0] = lW[0][1] - lW[1][0]; lrr[1] = lW[0][2] - lW[2][0]; lrr[2] = lW[1][2] - lW[2][1];

  for (int c = 0; c < 6; ++c) { LOUT(A_TAU + c) = ltau0[c]; LOUT(A_INC + c) = linc0[c]; TMP(J_SR + c, i) = lsr[c]; }
  for (int c = 0; c < 3; ++c) { TMP(J_RR + c, i) = lrr[c]; TMP(J_XN + c, i) = lxn[c]; TMP(J_VN + c, i) = LIN(A_V + c, i); }
  LOUT(A_PLS) = lpls0;
  LOUT(A_SY) = lsy0;
  LOUT(A_T) = ltn + lT0;
  LOUT(A_DTDT) = K.thermal_solver ? dt * ltn : 0.0;
  TMP(J_RHON, i) = lrhon;
  QA(Q_G) += lG;
  QA(Q_CS) += lCs;
  QA(Q_EP) += lEp;
}

// ---------------------------------------------------------------- R2: rates + second kick + drift
__global__ void __launch_bounds__(BLOCK) k_adj_rates_drift(AdjPtrs A, DomainConst K) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K.N) return;
  const DevPtrs& S = A.S;
  size_t N = K.N;
  double dt = K.dt;
  if (icol(S, I_KIND, N, i) != 0) {
    for (int c = 0; c < 3; ++c) { TMP(J_VH + c, i) = 0.0; TMP(J_AH + c, i) = 0.0; LOUT(A_X + c) = 0.0; }
    TMP(J_DRHO, i) = 0.0; LOUT(A_RHO) = 0.0;
    return;
  }
  double xi[3] = {FE(C_X, i), FE(C_X + 1, i), FE(C_X + 2, i)};
  double vi[3] = {FE(C_V, i), FE(C_V + 1, i), FE(C_V + 2, i)};
  double hi = col(S, C_H, N, i), wi = FE(C_MRHO, i), rhoN = FE(C_RHO, i);
  double inv_hi = 1.0 / hi;
  double li[9];
  for (int c = 0; c < 6; ++c) li[c] = TMP(J_SR + c, i);
  for (int c = 0; c < 3; ++c) li[6 + c] = TMP(J_RR + c, i);
  double lx[3] = {TMP(J_XN, i), TMP(J_XN + 1, i), TMP(J_XN + 2, i)};
  double lv[3] = {TMP(J_VN, i), TMP(J_VN + 1, i), TMP(J_VN + 2, i)};
  double lrhon = TMP(J_RHON, i);
  double sumLT = 0.0;
  int len = S.row_len[i];
  for (int k = 0; k < len; ++k) {
    int j = nb_index(S.nbr[(size_t)k * N + i]);
    GeoD g;
    if (K.thermal_solver) {  // R1 formed this entry's end-state geometry
      g.x0 = xi[0] - FE(C_X, j); g.x1 = xi[1] - FE(C_X + 1, j); g.x2 = xi[2] - FE(C_X + 2, j);
      g.GK = A.gk_end[(size_t)k * N + i];
      g.dGr = A.dg_end[(size_t)k * N + i];
    } else {
      g = geo_d(xi, hi, inv_hi, FE(C_X, j), FE(C_X + 1, j), FE(C_X + 2, j), col(S, C_H, N, j));
    }
    double b0 = vi[0] - FE(C_V, j), b1 = vi[1] - FE(C_V + 1, j), b2 = vi[2] - FE(C_V + 2, j);
    double wj = FE(C_MRHO, j);
    double lj[9], L[9];
    for (int c = 0; c < 6; ++c) lj[c] = TMP(J_SR + c, j);
    for (int c = 0; c < 3; ++c) lj[6 + c] = TMP(J_RR + c, j);
    for (int c = 0; c < 9; ++c) L[c] = wj * li[c] + wi * lj[c];
    double x0 = g.x0, x1 = g.x1, x2 = g.x2;
    double B[9] = {2.0 * b0 * x0, 2.0 * b1 * x1, 2.0 * b2 * x2, b0 * x1 + b1 * x0, b0 * x2 + b2 * x0,
                   b1 * x2 + b2 * x1, b0 * x1 - b1 * x0, b0 * x2 - b2 * x0, b1 * x2 - b2 * x1};
    double Q = 0.0, Qj = 0.0;
    for (int c = 0; c < 9; ++c) { Q += L[c] * B[c]; Qj += lj[c] * B[c]; }
    double f = -0.5 * g.GK;
    sumLT += f * Qj;
    double db0 = 2.0 * L[0] * x0 + L[3] * x1 + L[4] * x2 + L[6] * x1 + L[7] * x2;
    double db1 = 2.0 * L[1] * x1 + L[3] * x0 + L[5] * x2 - L[6] * x0 + L[8] * x2;
    double db2 = 2.0 * L[2] * x2 + L[4] * x0 + L[5] * x1 - L[7] * x0 - L[8] * x1;
    double dx0 = 2.0 * L[0] * b0 + L[3] * b1 + L[4] * b2 - L[6] * b1 - L[7] * b2;
    double dx1 = 2.0 * L[1] * b1 + L[3] * b0 + L[5] * b2 + L[6] * b0 - L[8] * b2;
    double dx2 = 2.0 * L[2] * b2 + L[4] * b0 + L[5] * b1 + L[7] * b0 + L[8] * b1;
    double gq = -0.5 * Q * g.dGr;
    lv[0] += f * db0; lv[1] += f * db1; lv[2] += f * db2;
    lx[0] += f * dx0 + gq * x0; lx[1] += f * dx1 + gq * x1; lx[2] += f * dx2 + gq * x2;
  }
  lrhon += -(wi / rhoN) * sumLT;
  double vb[3];
  bool isbc = bc_value(S.tab, icol(S, I_ID, N, i), A.time, vb);
  for (int d = 0; d < 3; ++d) {
    double lvpp = isbc ? 0.0 : lv[d];  // v' = vh + a2 dt/2 unless the BC overwrote it
    TMP(J_VH + d, i) = lvpp + dt * lx[d];
    TMP(J_AH + d, i) = lvpp * dt / 2.;
    LOUT(A_X + d) = lx[d];
  }
  LOUT(A_RHO) = lrhon;
  TMP(J_DRHO, i) = dt * lrhon;
}

// ---------------------------------------------------------------- R3: density + first kick + contact
__global__ void __launch_bounds__(BLOCK) k_adj_density_contact(AdjPtrs A, DomainConst K) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K.N) return;
  const DevPtrs& S = A.S;
  size_t N = K.N;
  double dt = K.dt;
  if (icol(S, I_KIND, N, i) != 0) {
    for (int c = 0; c < 3; ++c) { TMP(J_AACC + c, i) = 0.0; LOUT(A_V + c) = 0.0; }
    return;
  }
  double xi[3] = {col(S, C_X, N, i), col(S, C_X + 1, N, i), col(S, C_X + 2, N, i)};
  double vh[3] = {TXV(TX_VH, i), TXV(TX_VH + 1, i), TXV(TX_VH + 2, i)};
  double hi = col(S, C_H, N, i), rhoi = col(S, C_RHO, N, i), wi = col(S, C_MRHO, N, i);
  double inv_hi = 1.0 / hi, w_rho = -wi / rhoi;
  double ldr = TMP(J_DRHO, i);
  double lvh[3] = {TMP(J_VH, i), TMP(J_VH + 1, i), TMP(J_VH + 2, i)};
  double lx[3] = {0, 0, 0}, lrho = 0.0, D = 0.0;
  int len = S.row_len[i];
  for (int k = 0; k < len; ++k) {
    int j = nb_index(S.nbr[(size_t)k * N + i]);
    GeoD g = geo_d(xi, hi, inv_hi, col(S, C_X, N, j), col(S, C_X + 1, N, j), col(S, C_X + 2, N, j), col(S, C_H, N, j));
    A.gk_start[(size_t)k * N + i] = g.GK;  // R4 reads the same start-state geometry
    A.dg_start[(size_t)k * N + i] = g.dGr;
    double b0 = vh[0] - TXV(TX_VH, j), b1 = vh[1] - TXV(TX_VH + 1, j), b2 = vh[2] - TXV(TX_VH + 2, j);
    double bx = b0 * g.x0 + b1 * g.x1 + b2 * g.x2;
    double pd = g.GK * bx;
    double wj = col(S, C_MRHO, N, j), rhoj = col(S, C_RHO, N, j), ldj = TMP(J_DRHO, j);
    D += wj * pd;
    double Lam = ldr * rhoi * wj + ldj * rhoj * wi;
    lvh[0] += Lam * g.GK * g.x0; lvh[1] += Lam * g.GK * g.x1; lvh[2] += Lam * g.GK * g.x2;
    double c = Lam * bx * g.dGr;
    lx[0] += Lam * g.GK * b0 + c * g.x0; lx[1] += Lam * g.GK * b1 + c * g.x1; lx[2] += Lam * g.GK * b2 + c * g.x2;
    lrho += ldj * rhoj * w_rho * pd;
  }
  lrho += ldr * D;
  // second BC pass and the first half kick vh = v1 + a1 dt/2
  double vbi[3];
  bool isbc = bc_value(S.tab, icol(S, I_ID, N, i), A.time, vbi);
  double lv1[3], la[3];
  for (int d = 0; d < 3; ++d) {
    lv1[d] = isbc ? 0.0 : lvh[d];
    la[d] = isbc ? 0.0 : TMP(J_AH + d, i) + lvh[d] * 0.5 * dt;
  }
  // contact pairs of this particle, replayed then reversed (Contact_Wang.cpp:15-348)
  int ncp = K.contact ? S.cp_len[i] : 0;
  if (ncp > 0) {
    double x[3] = {xi[0], xi[1], xi[2]};
    double v[3];
    for (int d = 0; d < 3; ++d) v[d] = isbc ? vbi[d] : col(S, C_V + d, N, i);
    double m1 = col(S, C_MASS, N, i), h1 = hi;
    double a[3] = {TXV(TX_APRE, i), TXV(TX_APRE + 1, i), TXV(TX_APRE + 2, i)};
    int kin[ADJ_MAX_INSIDE];
    double ain[ADJ_MAX_INSIDE][3];
    int nin = 0;
    // geometry of pair k (mesh particle p2): normal, velocity after the first BC pass, plane, mesh
    auto pair_data = [&](int k, double n2[3], double v2[3], int& e, int& mm) {
      int p2 = S.cp[(size_t)k * N + i];
      for (int d = 0; d < 3; ++d) { n2[d] = col(S, C_NORMAL + d, N, p2); v2[d] = col(S, C_V + d, N, p2); }
      double vb2[3];
      if (bc_value(S.tab, icol(S, I_ID, N, p2), A.time, vb2)) for (int d = 0; d < 3; ++d) v2[d] = vb2[d];
      e = icol(S, I_ELEM, N, p2);
      mm = icol(S, I_MESH, N, p2);
    };
    auto kij_of = [&](double& base) {
      if (K.contact_alg == 1) {
        double r0 = col(S, C_RHO0, N, i), cs = col(S, C_CS, N, i), G = col(S, C_G, N, i);
        double bulk = cs * cs * r0;
        base = 9. * bulk * G / (3. * bulk + G) * pow(m1 / r0, 0.33333);
        return K.PFAC * base;
      } else if (K.contact_alg == 2) {
        base = pow(m1 / rhoi, 2.0 / 3.0);
        return K.PFAC * base;
      }
      base = 0.0;
      return 2.0 * m1 / (dt * dt);
    };
    for (int k = 0; k < ncp; ++k) {
      double n2[3], v2[3];
      int e, mm;
      pair_data(k, n2, v2, e, mm);
      double xp[3];
      for (int d = 0; d < 3; ++d) xp[d] = x[d] + v[d] * dt + a[d] * dt * dt / 2.0;
      double dist = n2[0] * xp[0] + n2[1] * xp[1] + n2[2] * xp[2] - S.elem_pplane[e];
      if (!(dist < h1)) continue;
      double qj[3] = {x[0] - dist * n2[0], x[1] - dist * n2[1], x[2] - dist * n2[2]};
      bool inside = true;
      for (int ii = 0; ii < 3 && inside; ++ii) {
        int jj = ii + 1; if (jj > 2) jj = 0;
        int na = S.elem_node[3 * e + ii], nb = S.elem_node[3 * e + jj];
        double pa[3] = {S.node[na], S.node[S.nnodes + na], S.node[2 * S.nnodes + na]};
        double pb[3] = {S.node[nb], S.node[S.nnodes + nb], S.node[2 * S.nnodes + nb]};
        double u[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
        double w[3] = {qj[0] - pa[0], qj[1] - pa[1], qj[2] - pa[2]};
        double cr[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
        if (cr[0] * n2[0] + cr[1] * n2[1] + cr[2] * n2[2] < 0.0) inside = false;
      }
      if (!inside) continue;
      if (nin == ADJ_MAX_INSIDE) { atomicOr(A.err, ERR_ADJ_CONTACT); break; }
      kin[nin] = k;
      for (int d = 0; d < 3; ++d) ain[nin][d] = a[d];
      ++nin;
      // forward update of a (same arithmetic as the step)
      double base;
      double kij = kij_of(base);
      double delta = h1 - dist;
      double vr[3] = {v[0] - v2[0], v[1] - v2[1], v[2] - v2[2]};
      double delta_ = -(n2[0] * vr[0] + n2[1] * vr[1] + n2[2] * vr[2]);
      double omega = sqrt(kij / m1);
      double psi = 2. * m1 * omega * K.DFAC;
      double s = kij * delta - psi * delta_;
      double cf[3];
      for (int d = 0; d < 3; ++d) { cf[d] = s * n2[d]; a[d] = a[d] + cf[d] / m1; }
      if (K.friction_sta > 0.) {
        double du[3];
        for (int d = 0; d < 3; ++d) du[d] = (xp[d] - x[d]) - v2[d] * dt;
        double dn = du[0] * n2[0] + du[1] * n2[1] + du[2] * n2[2];
        double tg[3];
        for (int d = 0; d < 3; ++d) tg[d] = kij * (du[d] - dn * n2[d]);
        double ntg = sqrt(tg[0] * tg[0] + tg[1] * tg[1] + tg[2] * tg[2]);
        double ncf = sqrt(cf[0] * cf[0] + cf[1] * cf[1] + cf[2] * cf[2]);
        if (ntg < K.friction_sta * ncf) {
          for (int d = 0; d < 3; ++d) a[d] -= tg[d] / m1;
        } else {
          double fs = K.friction_dyn * ncf;
          for (int d = 0; d < 3; ++d) a[d] -= fs * tg[d] / ntg / m1;
        }
      }
    }
    double lq_mu = 0.0, lq_pfac = 0.0, lq_g = 0.0, lq_cs = 0.0;
    double lvc[3] = {0, 0, 0};
    for (int r = nin - 1; r >= 0; --r) {
      int k = kin[r];
      double n2[3], v2[3];
      int e, mm;
      pair_data(k, n2, v2, e, mm);
      const double* a0 = ain[r];
      double xp[3];
      for (int d = 0; d < 3; ++d) xp[d] = x[d] + v[d] * dt + a0[d] * dt * dt / 2.0;
      double dist = n2[0] * xp[0] + n2[1] * xp[1] + n2[2] * xp[2] - S.elem_pplane[e];
      double base;
      double kij = kij_of(base);
      double delta = h1 - dist;
      double vr[3] = {v[0] - v2[0], v[1] - v2[1], v[2] - v2[2]};
      double delta_ = -(n2[0] * vr[0] + n2[1] * vr[1] + n2[2] * vr[2]);
      double omega = sqrt(kij / m1);
      double psi = 2. * m1 * omega * K.DFAC;
      double s = kij * delta - psi * delta_;
      double cfn[3] = {s * n2[0], s * n2[1], s * n2[2]};
      double lcf[3] = {0, 0, 0};
      if (mm == A.seed_mesh) for (int d = 0; d < 3; ++d) lcf[d] = A.seed[d];
      double lcfn[3] = {lcf[0] + la[0] / m1, lcf[1] + la[1] / m1, lcf[2] + la[2] / m1};
      double lxp[3] = {0, 0, 0}, lkij = 0.0;
      if (K.friction_sta > 0.) {
        double du[3];
        for (int d = 0; d < 3; ++d) du[d] = (xp[d] - x[d]) - v2[d] * dt;
        double dn = du[0] * n2[0] + du[1] * n2[1] + du[2] * n2[2];
        double dtg[3], tg[3];
        for (int d = 0; d < 3; ++d) { dtg[d] = du[d] - dn * n2[d]; tg[d] = kij * dtg[d]; }
        double ntg = sqrt(tg[0] * tg[0] + tg[1] * tg[1] + tg[2] * tg[2]);
        double ncf = sqrt(cfn[0] * cfn[0] + cfn[1] * cfn[1] + cfn[2] * cfn[2]);
        double ltg[3];
        if (ntg < K.friction_sta * ncf) {  // cf -= tg/m, a -= tg/m
          for (int d = 0; d < 3; ++d) ltg[d] = -(lcf[d] + la[d]) / m1;
        } else {  // td = mu_d |cf| tg/|tg|; cf -= td, a -= td/m
          double fs = K.friction_dyn * ncf;
          double th[3] = {tg[0] / ntg, tg[1] / ntg, tg[2] / ntg};
          double ltd[3], lfs = 0.0;
          for (int d = 0; d < 3; ++d) { ltd[d] = -lcf[d] - la[d] / m1; lfs += ltd[d] * th[d]; }
          for (int d = 0; d < 3; ++d) ltg[d] = fs * (ltd[d] - lfs * th[d]) / ntg;
          lq_mu += ncf * lfs;
          double lncf = K.friction_dyn * lfs;
          if (ncf > 0.0) for (int d = 0; d < 3; ++d) lcfn[d] += lncf * cfn[d] / ncf;
        }
        double ldtg[3];
        for (int d = 0; d < 3; ++d) { lkij += ltg[d] * dtg[d]; ldtg[d] = kij * ltg[d]; }
        double ldn = ldtg[0] * n2[0] + ldtg[1] * n2[1] + ldtg[2] * n2[2];
        for (int d = 0; d < 3; ++d) {
          double ldu = ldtg[d] - ldn * n2[d];
          lxp[d] += ldu;
          lx[d] -= ldu;
        }
      }
      // cf_n = s n2, s = kij delta - psi delta_
      double ls = lcfn[0] * n2[0] + lcfn[1] * n2[1] + lcfn[2] * n2[2];
      lkij += ls * delta;
      double ldelta = ls * kij;
      double ldelta_ = -ls * psi;
      if (K.DFAC != 0.0 && omega > 0.0) lkij += -ls * delta_ * K.DFAC / omega;
      for (int d = 0; d < 3; ++d) lvc[d] -= ldelta_ * n2[d];
      for (int d = 0; d < 3; ++d) lxp[d] += -ldelta * n2[d];
      for (int d = 0; d < 3; ++d) { lx[d] += lxp[d]; lvc[d] += dt * lxp[d]; la[d] += dt * dt / 2.0 * lxp[d]; }
      if (K.contact_alg == 2) {
        lq_pfac += lkij * base;
        lrho += -(2.0 / 3.0) * lkij * kij / rhoi;
      } else if (K.contact_alg == 1) {
        lq_pfac += lkij * base;
        double r0 = col(S, C_RHO0, N, i), cs = col(S, C_CS, N, i), G = col(S, C_G, N, i);
        double bulk = cs * cs * r0, den = 3. * bulk + G;
        double dS = pow(m1 / r0, 0.33333);
        double lb = lkij * K.PFAC * 9. * dS;
        lq_g += lb * 3. * bulk * bulk / (den * den);
        lq_cs += lb * G * G / (den * den) * 2.0 * cs * r0;
      }
    }
    if (!isbc) for (int d = 0; d < 3; ++d) lv1[d] += lvc[d];
    QA(Q_MU) += lq_mu;
    QA(Q_PFAC) += lq_pfac;
    QA(Q_G) += lq_g;
    QA(Q_CS) += lq_cs;
  }
  // first BC pass: a0 = 0 and v1 = v_bc for BC particles
  for (int d = 0; d < 3; ++d) {
    TMP(J_AACC + d, i) = isbc ? 0.0 : la[d];
    LOUT(A_V + d) = lv1[d];
    LOUT(A_X + d) += lx[d];
  }
  LOUT(A_RHO) += lrho;
}

// ---------------------------------------------------------------- R4: acceleration
__global__ void __launch_bounds__(BLOCK) k_adj_accel(AdjPtrs A, DomainConst K) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K.N) return;
  const DevPtrs& S = A.S;
  size_t N = K.N;
  if (icol(S, I_KIND, N, i) != 0) {
    for (int c = 0; c < 6; ++c) LOUT(A_SIG + c) = 0.0;
    return;
  }
  double xi[3] = {col(S, C_X, N, i), col(S, C_X + 1, N, i), col(S, C_X + 2, N, i)};
  double vi[3] = {col(S, C_V, N, i), col(S, C_V + 1, N, i), col(S, C_V + 2, N, i)};
  double hi = col(S, C_H, N, i), rhoi = col(S, C_RHO, N, i), csi = col(S, C_CS, N, i), mi = col(S, C_MASS, N, i);
  double al = col(S, C_ALPHA, N, i), be = col(S, C_BETA, N, i);
  double Si[6];
  for (int c = 0; c < 6; ++c) Si[c] = col(S, C_SRHO + c, N, i);
  double lai[3] = {TMP(J_AACC, i), TMP(J_AACC + 1, i), TMP(J_AACC + 2, i)};
  double lx[3] = {0, 0, 0}, lv[3] = {0, 0, 0}, lrho = 0.0, lcs = 0.0;
  double lSs[6] = {0, 0, 0, 0, 0, 0};
  int len = S.row_len[i];
  for (int k = 0; k < len; ++k) {
    int j = nb_index(S.nbr[(size_t)k * N + i]);
    double mj = col(S, C_MASS, N, j);
    double Gm[3];
    for (int d = 0; d < 3; ++d) Gm[d] = mj * lai[d] - mi * TMP(J_AACC + d, j);
    GeoD g;  // R3 formed this entry's start-state geometry
    g.x0 = xi[0] - col(S, C_X, N, j); g.x1 = xi[1] - col(S, C_X + 1, N, j); g.x2 = xi[2] - col(S, C_X + 2, N, j);
    g.GK = A.gk_start[(size_t)k * N + i];
    g.dGr = A.dg_start[(size_t)k * N + i];
    double b0 = vi[0] - col(S, C_V, N, j), b1 = vi[1] - col(S, C_V + 1, N, j), b2 = vi[2] - col(S, C_V + 2, N, j);
    double Alpha = K.av_uniform ? al : (al + col(S, C_ALPHA, N, j)) / 2.0;
    double Beta = K.av_uniform ? be : (be + col(S, C_BETA, N, j)) / 2.0;
    double PIs = 0.0, MU = 0.0, iDn = 0.0, Cij = 0.0, irbar = 0.0, hh = 0.0;
    bool av = false;
    if (Alpha != 0.0 || Beta != 0.0) {
      double dvx = b0 * g.x0 + b1 * g.x1 + b2 * g.x2;
      if (dvx < 0) {
        hh = (hi + col(S, C_H, N, j)) / 2;
        iDn = 1.0 / (g.x0 * g.x0 + g.x1 * g.x1 + g.x2 * g.x2 + 0.01 * hh * hh);
        MU = hh * dvx * iDn;
        Cij = 0.5 * (csi + col(S, C_CS, N, j));
        irbar = 2.0 / (rhoi + col(S, C_RHO, N, j));
        PIs = (Alpha * Cij * MU + Beta * MU * MU) * irbar;
        av = true;
      }
    }
    double S6[6];
    for (int c = 0; c < 6; ++c) S6[c] = Si[c] + col(S, C_SRHO + c, N, j) + (c < 3 ? PIs : 0.0);
    // pair contribution Gm . (GK x S) = GK x.(S Gm)
    double u0 = S6[0] * Gm[0] + S6[3] * Gm[1] + S6[4] * Gm[2];
    double u1 = S6[3] * Gm[0] + S6[1] * Gm[1] + S6[5] * Gm[2];
    double u2 = S6[4] * Gm[0] + S6[5] * Gm[1] + S6[2] * Gm[2];
    double xu = g.x0 * u0 + g.x1 * u1 + g.x2 * u2;
    lx[0] += g.GK * u0 + xu * g.dGr * g.x0;
    lx[1] += g.GK * u1 + xu * g.dGr * g.x1;
    lx[2] += g.GK * u2 + xu * g.dGr * g.x2;
    double gx0 = g.GK * g.x0, gx1 = g.GK * g.x1, gx2 = g.GK * g.x2;
    lSs[0] += gx0 * Gm[0]; lSs[1] += gx1 * Gm[1]; lSs[2] += gx2 * Gm[2];
    lSs[3] += gx0 * Gm[1]; lSs[3] += gx1 * Gm[0];
    lSs[4] += gx0 * Gm[2]; lSs[4] += gx2 * Gm[0];
    lSs[5] += gx1 * Gm[2]; lSs[5] += gx2 * Gm[1];
    if (av) {
      double lPI = gx0 * Gm[0] + gx1 * Gm[1] + gx2 * Gm[2];
      double lMU = lPI * (Alpha * Cij + 2.0 * Beta * MU) * irbar;
      lcs += lPI * Alpha * MU * irbar * 0.5;
      lrho += -lPI * PIs * irbar * 0.5;
      double cb = lMU * hh * iDn, cx = -lMU * 2.0 * MU * iDn;
      lx[0] += cb * b0 + cx * g.x0; lx[1] += cb * b1 + cx * g.x1; lx[2] += cb * b2 + cx * g.x2;
      lv[0] += cb * g.x0; lv[1] += cb * g.x1; lv[2] += cb * g.x2;
    }
  }
  // S_i = Sigma_i / rho_i^2
  double inv2 = 1.0 / (rhoi * rhoi);
  double ls = 0.0;
  for (int c = 0; c < 6; ++c) { LOUT(A_SIG + c) = lSs[c] * inv2; ls += lSs[c] * Si[c]; }
  lrho += -2.0 / rhoi * ls;
  for (int d = 0; d < 3; ++d) { LOUT(A_X + d) += lx[d]; LOUT(A_V + d) += lv[d]; }
  LOUT(A_RHO) += lrho;
  QA(Q_CS) += lcs;
}

// ---------------------------------------------------------------- bookkeeping
__global__ void k_unpermute(const int* perm, const double* src, double* dst, int ncol, int N) {
  size_t total = (size_t)ncol * N;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
    size_t c = k / N, p = k - c * N;
    dst[c * N + perm[p]] = src[k];
  }
}

// Initial Sigmay (CalcYieldStress(0, 0, T0) for Johnson-Cook particles,
// WeldForm.cpp:905-906; the given value otherwise), the chain rule of E into
// G = E / (2 (1 + nu)) and Cs = sqrt(E / (3 (1 - 2 nu) rho0)), and one block
// partial sum per parameter.
__global__ void k_adj_finish(DevPtrs P, DomainConst K, const double* L, double* Q, double* partials) {
  __shared__ double sh[32];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  size_t N = K.N;
  double g[ADJ_NPARAM];
  for (int p = 0; p < ADJ_NPARAM; ++p) g[p] = 0.0;
  if (i < K.N && icol(P, I_KIND, N, i) == 0) {
    auto q = [&](int c) { return Q[(size_t)c * N + i]; };
    int mi = icol(P, I_MAT, N, i), model = icol(P, I_MODEL, N, i);
    const MaterialDev* M = (mi >= 0 && mi < P.tab->nmat) ? &P.tab->mat[mi] : nullptr;
    double lsy = L[(size_t)A_SY * N + i];
    double qA = q(Q_A), qM = q(Q_M), qS = q(Q_SY0);
    if (model == 2 && M) {
      double Th = (col(P, C_T, N, i) - M->T_t) / (M->T_m - M->T_t);
      double Thm = pow(Th, M->jm);
      qA += lsy * (1.0 - Thm);
      if (Th > 0.0) qM += -lsy * M->A * Thm * log(Th);
    } else {
      qS += lsy;
    }
    if (M && M->E != 0.0) g[0] = (q(Q_G) * col(P, C_G, N, i) + q(Q_CS) * col(P, C_CS, N, i) * 0.5) / M->E;
    g[1] = qS; g[2] = q(Q_EP); g[3] = qA; g[4] = q(Q_B); g[5] = q(Q_N); g[6] = q(Q_C); g[7] = qM;
    g[8] = q(Q_MU); g[9] = q(Q_PFAC);
  }
  for (int p = 0; p < ADJ_NPARAM; ++p) {
    double r = block_reduce<0>(g[p], sh);
    if (threadIdx.x == 0) partials[(size_t)p * gridDim.x + blockIdx.x] = r;
  }
}
__global__ void k_adj_sum(const double* partials, int nb, double* out) {
  __shared__ double sh[256];
  int p = blockIdx.x;
  double acc = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) acc += partials[(size_t)p * nb + b];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[p] = sh[0];
}

__global__ void k_record_force(const StepState* st, int mesh, int axis, double* out, long long n) {
  if (threadIdx.x == 0 && blockIdx.x == 0) out[n] = st->contact_force[mesh][axis];
}

// Per-particle factor of the conduction adjoint, d loss / d dTdt' / (rho' cp),
// read by both ends of every pair in R1.
__global__ void k_adj_conduction_factor(AdjPtrs A, DomainConst K) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K.N) return;
  const DevPtrs& S = A.S;
  size_t N = K.N;
  TMP(J_LC, i) = icol(S, I_KIND, N, i) == 0 ? LIN(A_DTDT, i) / (FE(C_RHO, i) * col(S, C_CPT, N, i)) : 0.0;
}

void launch_adjoint_step(const AdjPtrs& A, const DomainConst& K, cudaStream_t s) {
  // one thread per particle, no block-level sums: the domain's per-particle block size
  int tb = K.pblock > 0 ? K.pblock : BLOCK;
  int nb = nblk(K.N, tb);
  if (K.thermal_solver) {
    k_adj_conduction_factor<<<nb, tb, 0, s>>>(A, K);
    mark(s, "k_adj_conduction_factor");
  }
  k_adj_thermal_stress<<<nb, tb, 0, s>>>(A, K);
  mark(s, "k_adj_thermal_stress");
  k_adj_rates_drift<<<nb, tb, 0, s>>>(A, K);
  mark(s, "k_adj_rates_drift");
  k_adj_density_contact<<<nb, tb, 0, s>>>(A, K);
  mark(s, "k_adj_density_contact");
  k_adj_accel<<<nb, tb, 0, s>>>(A, K);
  mark(s, "k_adj_accel");
}
void launch_unpermute(const int* perm, const double* src, double* dst, int ncol, int N, cudaStream_t s) {
  k_unpermute<<<152 * 4, 512, 0, s>>>(perm, src, dst, ncol, N);
  mark(s, "k_unpermute");
}
void launch_adjoint_finish(const DevPtrs& P0, const DomainConst& K, const double* Lstart, double* Q, double* partials,
                           double* out, cudaStream_t s) {
  int nb = nblk(K.N, BLOCK);
  k_adj_finish<<<nb, BLOCK, 0, s>>>(P0, K, Lstart, Q, partials);
  k_adj_sum<<<ADJ_NPARAM, 256, 0, s>>>(partials, nb, out);
}
void launch_record_force(const DevPtrs& P, int mesh, int axis, double* out, long long n, cudaStream_t s) {
  k_record_force<<<1, 32, 0, s>>>(P.st, mesh, axis, out, n);
}

}  // namespace wf
