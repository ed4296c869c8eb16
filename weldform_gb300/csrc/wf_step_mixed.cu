// Mixed FP32/FP64 form of the kick-drift step on sm_103a.
//
// Same launch sequence and reference semantics as the plain form
// (wf_step_fp64.cu); what changes is the arithmetic of the pair gathers:
//  * relative positions, velocities and temperatures are formed from
//    float-float shadows (hi = fl(v), lo = fl(v - hi)) as
//    (hi_i - hi_j) + (lo_i - lo_j): accurate to FP32 rounding of the
//    difference itself, the accuracy an FP64 difference cast to FP32 has, with
//    FP32 instructions only (GB300 issues FP64 at 1/72 of its FP32 rate);
//  * kernel gradients, viscosity and pair terms in FP32;
//  * every per-particle pair sum is Kahan-compensated in FP32;
//  * FP64 stays in: position/velocity/density integration, the stress
//    accumulation and its radial-return yield check and scale factor, the
//    temperature update, and all global reductions.
#include "wf_step_common.cuh"
#include "wf_launch.h"

namespace wf {

static inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

constexpr float INV_PI_F = 0.318309886183790671538f;

// Kahan-compensated FP32 sum; value() = s - c.
struct KSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// Pair geometry in FP32 from float-float positions.  GK as in
// Functions.cpp:74-87 (cubic spline, 3D).
struct GeoF {
  float x0, x1, x2, r2, r, hh, GK;
};
__device__ __forceinline__ GeoF geo_f(const DevPtrs& P, size_t N, int hcol, int lcol, float xh0, float xh1, float xh2,
                                      float xl0, float xl1, float xl2, float hi, int j) {
  GeoF g;
  g.x0 = (xh0 - P.g[(size_t)(hcol + 0) * N + j]) + (xl0 - P.g[(size_t)(lcol + 0) * N + j]);
  g.x1 = (xh1 - P.g[(size_t)(hcol + 1) * N + j]) + (xl1 - P.g[(size_t)(lcol + 1) * N + j]);
  g.x2 = (xh2 - P.g[(size_t)(hcol + 2) * N + j]) + (xl2 - P.g[(size_t)(lcol + 2) * N + j]);
  g.r2 = g.x0 * g.x0 + g.x1 * g.x1 + g.x2 * g.x2;
  float rinv = rsqrtf(g.r2);
  g.r = g.r2 * rinv;
  float hj = P.g[(size_t)G_H * N + j];
  g.hh = 0.5f * (hi + hj);
  float inv_h = 1.0f / g.hh;
  float q = g.r * inv_h;
  float ih2 = inv_h * inv_h;
  float C = INV_PI_F * ih2 * ih2;
  float w;
  if (q < 1.0f) w = -3.0f + 2.25f * q;
  else if (q < 2.0f) { float t = 2.0f - q; w = -0.75f * t * t * (g.hh * rinv); }
  else w = 0.0f;
  if (g.r2 == 0.0f) { w = -3.0f; g.r = 0.0f; }
  g.GK = C * inv_h * w;
  return g;
}

// ---------------------------------------------------------------- shadows
__global__ void k_refresh_shadows(DevPtrs P, DomainConst K, int force) {
  if (!force && !P.st->do_search) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K.N) return;
  size_t N = K.N;
  for (int d = 0; d < 3; ++d) {
    store_ff(P, G_XH + d, G_XL + d, N, i, col(P, C_X + d, N, i));
    store_ff(P, G_VH + d, G_VL + d, N, i, col(P, C_V + d, N, i));
  }
  store_ff(P, G_TH, G_TL, N, i, col(P, C_T, N, i));
  bool solid = icol(P, I_KIND, N, i) == 0;
  double rho = col(P, C_RHO, N, i);
  double c2 = solid ? 1.0 / (rho * rho) : 0.0;
  for (int c = 0; c < 6; ++c) gcol(P, G_SRHO + c, N, i) = (float)(c2 * col(P, C_SIG + c, N, i));
  gcol(P, G_MRHO, N, i) = solid ? (float)(col(P, C_MASS, N, i) / rho) : 0.f;
  gcol(P, G_RHO, N, i) = (float)rho;
  gcol(P, G_PR2, N, i) = (float)(c2 * col(P, C_P, N, i));
  gcol(P, G_H, N, i) = (float)col(P, C_H, N, i);
  gcol(P, G_M, N, i) = (float)col(P, C_MASS, N, i);
  gcol(P, G_CS, N, i) = (float)col(P, C_CS, N, i);
  gcol(P, G_ALPHA, N, i) = (float)col(P, C_ALPHA, N, i);
  gcol(P, G_BETA, N, i) = (float)col(P, C_BETA, N, i);
  gcol(P, G_KT, N, i) = (float)col(P, C_KT, N, i);
}

// ---------------------------------------------------------------- accel
__global__ void __launch_bounds__(BLOCK) k_accel_mx(DevPtrs P, DomainConst K) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K.N) return;
  size_t N = K.N;
  if (icol(P, I_KIND, N, i) != 0) {
    colw(P, C_A, N, i) = 0.0; colw(P, C_A + 1, N, i) = 0.0; colw(P, C_A + 2, N, i) = 0.0;
    return;
  }
  float xh0 = gcol(P, G_XH, N, i), xh1 = gcol(P, G_XH + 1, N, i), xh2 = gcol(P, G_XH + 2, N, i);
  float xl0 = gcol(P, G_XL, N, i), xl1 = gcol(P, G_XL + 1, N, i), xl2 = gcol(P, G_XL + 2, N, i);
  float vh0 = gcol(P, G_VH, N, i), vh1 = gcol(P, G_VH + 1, N, i), vh2 = gcol(P, G_VH + 2, N, i);
  float vl0 = gcol(P, G_VL, N, i), vl1 = gcol(P, G_VL + 1, N, i), vl2 = gcol(P, G_VL + 2, N, i);
  float hi = gcol(P, G_H, N, i), rhoi = gcol(P, G_RHO, N, i), csi = gcol(P, G_CS, N, i);
  float ai = gcol(P, G_ALPHA, N, i), bi = gcol(P, G_BETA, N, i);
  float Si[6];
  for (int c = 0; c < 6; ++c) Si[c] = gcol(P, G_SRHO + c, N, i);
  KSum a0, a1, a2;
  int len = P.row_len[i];
  for (int k = 0; k < len; ++k) {
    int j = P.nbr[(size_t)k * N + i];
    GeoF g = geo_f(P, N, G_XH, G_XL, xh0, xh1, xh2, xl0, xl1, xl2, hi, j);
    float Alpha = 0.5f * (ai + gcol(P, G_ALPHA, N, j)), Beta = 0.5f * (bi + gcol(P, G_BETA, N, j));
    float v0 = (vh0 - gcol(P, G_VH, N, j)) + (vl0 - gcol(P, G_VL, N, j));
    float v1 = (vh1 - gcol(P, G_VH + 1, N, j)) + (vl1 - gcol(P, G_VL + 1, N, j));
    float v2 = (vh2 - gcol(P, G_VH + 2, N, j)) + (vl2 - gcol(P, G_VL + 2, N, j));
    float PIs = 0.f;
    if (Alpha != 0.f || Beta != 0.f) {
      float dvx = v0 * g.x0 + v1 * g.x1 + v2 * g.x2;
      if (dvx < 0.f) {
        float MU = g.hh * dvx / (g.r * g.r + 0.01f * g.hh * g.hh);
        float Cij = 0.5f * (csi + gcol(P, G_CS, N, j));
        PIs = (Alpha * Cij * MU + Beta * MU * MU) / (0.5f * (rhoi + gcol(P, G_RHO, N, j)));
      }
    }
    float S0 = Si[0] + gcol(P, G_SRHO + 0, N, j) + PIs;
    float S1 = Si[1] + gcol(P, G_SRHO + 1, N, j) + PIs;
    float S2 = Si[2] + gcol(P, G_SRHO + 2, N, j) + PIs;
    float S3 = Si[3] + gcol(P, G_SRHO + 3, N, j);
    float S4 = Si[4] + gcol(P, G_SRHO + 4, N, j);
    float S5 = Si[5] + gcol(P, G_SRHO + 5, N, j);
    float g0 = g.GK * g.x0, g1 = g.GK * g.x1, g2 = g.GK * g.x2;
    float mj = gcol(P, G_M, N, j);
    a0.add(mj * (g0 * S0 + g1 * S3 + g2 * S4));
    a1.add(mj * (g0 * S3 + g1 * S1 + g2 * S5));
    a2.add(mj * (g0 * S4 + g1 * S5 + g2 * S2));
  }
  colw(P, C_A, N, i) = a0.value(); colw(P, C_A + 1, N, i) = a1.value(); colw(P, C_A + 2, N, i) = a2.value();
}

// ---------------------------------------------------------------- density + drift + kick
__global__ void __launch_bounds__(BLOCK) k_density_drift_mx(DevPtrs P, DomainConst K) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K.N) return;
  size_t N = K.N;
  double dt = K.dt;
  double rhoi = col(P, C_RHO, N, i);
  double dd = 0.0;
  bool solid = icol(P, I_KIND, N, i) == 0;
  if (solid) {
    float xh0 = gcol(P, G_XH, N, i), xh1 = gcol(P, G_XH + 1, N, i), xh2 = gcol(P, G_XH + 2, N, i);
    float xl0 = gcol(P, G_XL, N, i), xl1 = gcol(P, G_XL + 1, N, i), xl2 = gcol(P, G_XL + 2, N, i);
    float vh0 = gcol(P, G_VH, N, i), vh1 = gcol(P, G_VH + 1, N, i), vh2 = gcol(P, G_VH + 2, N, i);
    float vl0 = gcol(P, G_VL, N, i), vl1 = gcol(P, G_VL + 1, N, i), vl2 = gcol(P, G_VL + 2, N, i);
    float hi = gcol(P, G_H, N, i);
    KSum s;
    int len = P.row_len[i];
    for (int k = 0; k < len; ++k) {
      int j = P.nbr[(size_t)k * N + i];
      GeoF g = geo_f(P, N, G_XH, G_XL, xh0, xh1, xh2, xl0, xl1, xl2, hi, j);
      float v0 = (vh0 - gcol(P, G_VH, N, j)) + (vl0 - gcol(P, G_VL, N, j));
      float v1 = (vh1 - gcol(P, G_VH + 1, N, j)) + (vl1 - gcol(P, G_VL + 1, N, j));
      float v2 = (vh2 - gcol(P, G_VH + 2, N, j)) + (vl2 - gcol(P, G_VL + 2, N, j));
      s.add(gcol(P, G_MRHO, N, j) * (g.GK * (v0 * g.x0 + v1 * g.x1 + v2 * g.x2)));
    }
    dd = s.value() * rhoi;
  }
  colw(P, C_DRHO, N, i) = dd;
  double rn = rhoi + dt * dd;
  colw(P, C_RHON, N, i) = rn;
  double mrn = solid ? col(P, C_MASS, N, i) / rn : 0.0;
  colw(P, C_MRHON, N, i) = mrn;
  gcol(P, G_MRHON, N, i) = (float)mrn;
  gcol(P, G_RHON, N, i) = (float)rn;
  for (int d = 0; d < 3; ++d) {
    double v = col(P, C_V + d, N, i);
    double du = v * dt;
    colw(P, C_DISP + d, N, i) = col(P, C_DISP + d, N, i) + du;
    double xn = col(P, C_X + d, N, i) + du;
    double vn = v + col(P, C_A + d, N, i) * dt / 2.;
    colw(P, C_XN + d, N, i) = xn;
    colw(P, C_VN + d, N, i) = vn;
    store_ff(P, G_XHN + d, G_XLN + d, N, i, xn);
    store_ff(P, G_VHN + d, G_VLN + d, N, i, vn);
  }
}

// ---------------------------------------------------------------- rate + stress
// Radial return with the Jaumann increment formed in FP32 and accumulated
// into the FP64 deviatoric stress; the yield check, scale factor and plastic
// strain increment are FP64 (Particle.cpp:960-1067).
__device__ __forceinline__ double stress_update_mx(StressIO& s, const float sr[6], const float rr[3], double rho,
                                                   double rho0, double Cs, double P0, double G, double T, int fail,
                                                   int model, const MaterialDev* M, double dt) {
  s.pressure = P0 + (Cs * Cs) * (rho - rho0);
  float S[3][3] = {{(float)s.tau[0], (float)s.tau[3], (float)s.tau[4]},
                   {(float)s.tau[3], (float)s.tau[1], (float)s.tau[5]},
                   {(float)s.tau[4], (float)s.tau[5], (float)s.tau[2]}};
  float W[3][3] = {{0.f, rr[0], rr[1]}, {-rr[0], 0.f, rr[2]}, {-rr[1], -rr[2], 0.f}};
  const int ui[6] = {0, 1, 2, 0, 0, 1}, uj[6] = {0, 1, 2, 1, 2, 2};
  float s3 = (1.0f / 3.0f) * (sr[0] + sr[1] + sr[2]);
  float twoG = (float)(2.0 * G), dtf = (float)dt;
  double t6[6];
  for (int c = 0; c < 6; ++c) {
    int a = ui[c], b = uj[c];
    float srt = S[a][2] * W[b][2] + S[a][1] * W[b][1] + S[a][0] * W[b][0];
    float rs = W[a][2] * S[2][b] + W[a][1] * S[1][b] + W[a][0] * S[0][b];
    float dev = sr[c] - (c < 3 ? s3 : 0.f);
    float inc = dtf * (twoG * dev + srt + rs);
    t6[c] = s.tau[c] + (double)inc;
  }
  float d01 = sr[0] - sr[1], d12 = sr[1] - sr[2], d20 = sr[2] - sr[0];
  float esr = sqrtf(0.5f * (d01 * d01 + d12 * d12 + d20 * d20) + 3.0f * (sr[3] * sr[3] + sr[5] * sr[5] + sr[4] * sr[4]));
  s.esr = esr;
  double dep = 0.0;
  if (fail == 1) {
    double J2 = 0.5 * (t6[0] * t6[0] + 2.0 * t6[3] * t6[3] + 2.0 * t6[4] * t6[4] + t6[1] * t6[1] +
                       2.0 * t6[5] * t6[5] + t6[2] * t6[2]);
    double sig_trial = sqrt(3.0 * J2);
    double ratio = s.sigmay / sig_trial;
    double sc = (1.0 < ratio) ? 1.0 : ratio;
    if (sc < 1.0)
      for (int c = 0; c < 6; ++c) t6[c] = sc * t6[c];
    if (model == 1 && M) {
      s.sigmay = (double)(M->K * powf((float)(s.pl_strain + M->eps0), (float)M->m));
      if (!(s.pl_strain + M->eps0 > M->eps1)) s.sigmay = M->sy0;
    } else if (model == 2 && M) {
      float Th = (float)((T - M->T_t) / (M->T_m - M->T_t));
      float f = 1.0f;
      if (esr > (float)M->eps_0) f = 1.0f + (float)M->C * logf(esr / (float)M->eps_0);
      s.sigmay = (double)(((float)M->A + (float)M->B * powf((float)s.pl_strain, (float)M->n)) * f *
                          (1.0f - powf(Th, (float)M->jm)));
    }
    if (sig_trial > s.sigmay) {
      if (s.Ep < 0) s.Ep = M ? M->E : 0.0;
      dep = (sig_trial - s.sigmay) / (3. * G + s.Ep);
      s.pl_strain += dep;
      s.delta_pl_strain = dep;
      if (model == 0) s.sigmay += dep * s.Ep;
    }
  }
  for (int c = 0; c < 6; ++c) s.tau[c] = t6[c];
  for (int c = 0; c < 6; ++c) s.sig[c] = (c < 3 ? -s.pressure : 0.0) + t6[c];
  if (dep > 0.0) {
    double f = dep / s.sigmay;
    s.epli[0] = f * (s.sig[0] - 0.5 * (s.sig[1] + s.sig[2]));
    s.epli[1] = f * (s.sig[1] - 0.5 * (s.sig[0] + s.sig[2]));
    s.epli[2] = f * (s.sig[2] - 0.5 * (s.sig[0] + s.sig[1]));
    s.epli[3] = 1.5 * f * s.sig[3];
    s.epli[4] = 1.5 * f * s.sig[4];
    s.epli[5] = 1.5 * f * s.sig[5];
    for (int c = 0; c < 6; ++c) s.epl[c] = s.epl[c] + s.epli[c];
  }
  for (int c = 0; c < 6; ++c) s.eps[c] = dt * (double)sr[c] + s.eps[c];
  return dep;
}

// Gather half: strain-rate and rotation-rate sums (InteractionAlt.cpp:263-479),
// written as float columns for the elementwise update below.  Kept lean so the
// gather runs at high occupancy.
__global__ void __launch_bounds__(BLOCK) k_rate_mx(DevPtrs P, DomainConst K, float* rates) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K.N) return;
  size_t N = K.N;
  float out[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (icol(P, I_KIND, N, i) == 0) {
    float xh0 = gcol(P, G_XHN, N, i), xh1 = gcol(P, G_XHN + 1, N, i), xh2 = gcol(P, G_XHN + 2, N, i);
    float xl0 = gcol(P, G_XLN, N, i), xl1 = gcol(P, G_XLN + 1, N, i), xl2 = gcol(P, G_XLN + 2, N, i);
    float vh0 = gcol(P, G_VHN, N, i), vh1 = gcol(P, G_VHN + 1, N, i), vh2 = gcol(P, G_VHN + 2, N, i);
    float vl0 = gcol(P, G_VLN, N, i), vl1 = gcol(P, G_VLN + 1, N, i), vl2 = gcol(P, G_VLN + 2, N, i);
    float hi = gcol(P, G_H, N, i);
    KSum M[9];  // sum_j (m_j/rho_j) (-GK/2) (v_i - v_j)_k (x_i - x_j)_l
    int len = P.row_len[i];
    for (int k = 0; k < len; ++k) {
      int j = P.nbr[(size_t)k * N + i];
      GeoF g = geo_f(P, N, G_XHN, G_XLN, xh0, xh1, xh2, xl0, xl1, xl2, hi, j);
      float b0 = (vh0 - gcol(P, G_VHN, N, j)) + (vl0 - gcol(P, G_VLN, N, j));
      float b1 = (vh1 - gcol(P, G_VHN + 1, N, j)) + (vl1 - gcol(P, G_VLN + 1, N, j));
      float b2 = (vh2 - gcol(P, G_VHN + 2, N, j)) + (vl2 - gcol(P, G_VLN + 2, N, j));
      float w = gcol(P, G_MRHON, N, j) * (-0.5f * g.GK);
      float wb0 = w * b0, wb1 = w * b1, wb2 = w * b2;
      M[0].add(wb0 * g.x0); M[1].add(wb0 * g.x1); M[2].add(wb0 * g.x2);
      M[3].add(wb1 * g.x0); M[4].add(wb1 * g.x1); M[5].add(wb1 * g.x2);
      M[6].add(wb2 * g.x0); M[7].add(wb2 * g.x1); M[8].add(wb2 * g.x2);
    }
    double m[9];
    for (int c = 0; c < 9; ++c) m[c] = M[c].value();
    // StrainRate = symmetric part (InteractionAlt.cpp:338-351), RotationRate
    // = antisymmetric part (355-361)
    out[0] = (float)(2.0 * m[0]); out[1] = (float)(2.0 * m[4]); out[2] = (float)(2.0 * m[8]);
    out[3] = (float)(m[1] + m[3]); out[4] = (float)(m[2] + m[6]); out[5] = (float)(m[5] + m[7]);
    out[6] = (float)(m[1] - m[3]); out[7] = (float)(m[2] - m[6]); out[8] = (float)(m[5] - m[7]);
  }
  for (int c = 0; c < 9; ++c) rates[(size_t)c * N + i] = out[c];
}

// Elementwise half: constitutive update, heating, temperature, and the
// next-step buffers becoming current.
__global__ void __launch_bounds__(BLOCK) k_stress_mx(DevPtrs P, DomainConst K, const float* rates) {
  __shared__ double sh[32];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  size_t N = K.N;
  double dt = K.dt;
  double plw = 0.0, maxpl = 0.0, maxT = -1e300, minT = 1e300;
  if (i < K.N) {
    for (int d = 0; d < 3; ++d) {
      colw(P, C_X + d, N, i) = col(P, C_XN + d, N, i);
      colw(P, C_V + d, N, i) = col(P, C_VN + d, N, i);
      gcol(P, G_XH + d, N, i) = gcol(P, G_XHN + d, N, i);
      gcol(P, G_XL + d, N, i) = gcol(P, G_XLN + d, N, i);
      gcol(P, G_VH + d, N, i) = gcol(P, G_VHN + d, N, i);
      gcol(P, G_VL + d, N, i) = gcol(P, G_VLN + d, N, i);
    }
    double rho = col(P, C_RHON, N, i);
    colw(P, C_RHO, N, i) = rho;
    colw(P, C_MRHO, N, i) = col(P, C_MRHON, N, i);
    gcol(P, G_MRHO, N, i) = gcol(P, G_MRHON, N, i);
    gcol(P, G_RHO, N, i) = gcol(P, G_RHON, N, i);
    maxpl = col(P, C_PLS, N, i);
    if (icol(P, I_KIND, N, i) == 0) {
      float sr[6], rr[3];
      for (int c = 0; c < 6; ++c) sr[c] = rates[(size_t)c * N + i];
      for (int c = 0; c < 3; ++c) rr[c] = rates[(size_t)(6 + c) * N + i];
      StressIO s;
      for (int c = 0; c < 6; ++c) {
        s.tau[c] = col(P, C_TAU + c, N, i); s.eps[c] = col(P, C_EPS + c, N, i);
        s.epl[c] = col(P, C_EPL + c, N, i); s.epli[c] = col(P, C_EPLI + c, N, i);
      }
      s.pl_strain = col(P, C_PLS, N, i); s.delta_pl_strain = col(P, C_DPLS, N, i);
      s.sigmay = col(P, C_SY, N, i); s.Ep = col(P, C_EP, N, i);
      int mi = icol(P, I_MAT, N, i);
      const MaterialDev* Mt = (mi >= 0 && mi < P.tab->nmat) ? &P.tab->mat[mi] : nullptr;
      double T = col(P, C_T, N, i);
      stress_update_mx(s, sr, rr, rho, col(P, C_RHO0, N, i), col(P, C_CS, N, i), col(P, C_P0, N, i),
                       col(P, C_G, N, i), T, icol(P, I_FAIL, N, i), icol(P, I_MODEL, N, i), Mt, dt);
      for (int c = 0; c < 6; ++c) {
        colw(P, C_TAU + c, N, i) = s.tau[c]; colw(P, C_SIG + c, N, i) = s.sig[c];
        colw(P, C_EPS + c, N, i) = s.eps[c]; colw(P, C_EPL + c, N, i) = s.epl[c];
        colw(P, C_EPLI + c, N, i) = s.epli[c]; colw(P, C_SR + c, N, i) = (double)sr[c];
      }
      for (int c = 0; c < 3; ++c) colw(P, C_RR + c, N, i) = (double)rr[c];
      colw(P, C_P, N, i) = s.pressure; colw(P, C_PLS, N, i) = s.pl_strain; colw(P, C_DPLS, N, i) = s.delta_pl_strain;
      colw(P, C_SY, N, i) = s.sigmay; colw(P, C_EP, N, i) = s.Ep; colw(P, C_ESR, N, i) = s.esr;
      maxpl = s.pl_strain;
      float c2 = 1.0f / ((float)rho * (float)rho);
      for (int c = 0; c < 6; ++c) gcol(P, G_SRHO + c, N, i) = c2 * (float)s.sig[c];
      gcol(P, G_PR2, N, i) = c2 * (float)s.pressure;
      if (K.pl_heating) {
        double q = col(P, C_QPL, N, i);
        if (s.delta_pl_strain > 0.0) q = plastic_heat(s.sig, s.epli, dt);
        colw(P, C_QPL, N, i) = q;
        colw(P, C_PSEN, N, i) = col(P, C_PSEN, N, i) + q * dt;
        plw = col(P, C_MASS, N, i) / rho * q;
      }
      if (K.thermal_solver) {
        T += dt * col(P, C_DTDT, N, i);
        colw(P, C_T, N, i) = T;
        store_ff(P, G_TH, G_TL, N, i, T);
        maxT = T; minT = T;
      }
    }
  }
  double r;
  r = block_reduce<1>(maxpl, sh); if (threadIdx.x == 0) P.partials[S_MAXPL * K.nblocks + blockIdx.x] = r;
  if (K.pl_heating) { r = block_reduce<0>(plw, sh); if (threadIdx.x == 0) P.partials[S_PLW * K.nblocks + blockIdx.x] = r; }
  if (K.thermal_solver) {
    r = block_reduce<1>(maxT, sh); if (threadIdx.x == 0) P.partials[S_MAXT * K.nblocks + blockIdx.x] = r;
    r = block_reduce<2>(minT, sh); if (threadIdx.x == 0) P.partials[S_MINT * K.nblocks + blockIdx.x] = r;
  }
}

// ---------------------------------------------------------------- energies (+ conduction)
__global__ void __launch_bounds__(BLOCK) k_energy_mx(DevPtrs P, DomainConst K) {
  __shared__ double sh[32];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  size_t N = K.N;
  double dkin = 0.0, dint = 0.0;
  if (i < K.N && icol(P, I_KIND, N, i) == 0) {
    float xh0 = gcol(P, G_XH, N, i), xh1 = gcol(P, G_XH + 1, N, i), xh2 = gcol(P, G_XH + 2, N, i);
    float xl0 = gcol(P, G_XL, N, i), xl1 = gcol(P, G_XL + 1, N, i), xl2 = gcol(P, G_XL + 2, N, i);
    float vh0 = gcol(P, G_VH, N, i), vh1 = gcol(P, G_VH + 1, N, i), vh2 = gcol(P, G_VH + 2, N, i);
    float vl0 = gcol(P, G_VL, N, i), vl1 = gcol(P, G_VL + 1, N, i), vl2 = gcol(P, G_VL + 2, N, i);
    float hi = gcol(P, G_H, N, i), mi = gcol(P, G_M, N, i), mrhoi = gcol(P, G_MRHO, N, i), pri = gcol(P, G_PR2, N, i);
    float thi = gcol(P, G_TH, N, i), tli = gcol(P, G_TL, N, i), ki = gcol(P, G_KT, N, i);
    KSum kin, cond;
    int len = P.row_len[i], split = P.row_split[i];
    for (int k = 0; k < len; ++k) {
      int j = P.nbr[(size_t)k * N + i];
      GeoF g = geo_f(P, N, G_XH, G_XL, xh0, xh1, xh2, xl0, xl1, xl2, hi, j);
      float b0 = (vh0 - gcol(P, G_VH, N, j)) + (vl0 - gcol(P, G_VL, N, j));
      float b1 = (vh1 - gcol(P, G_VH + 1, N, j)) + (vl1 - gcol(P, G_VL + 1, N, j));
      float b2 = (vh2 - gcol(P, G_VH + 2, N, j)) + (vl2 - gcol(P, G_VL + 2, N, j));
      float dv = g.GK * (b0 * g.x0 + b1 * g.x1 + b2 * g.x2);
      bool up = k < split;
      float pk = 0.5f * (up ? gcol(P, G_M, N, j) : mi) * (pri + gcol(P, G_PR2, N, j)) * dv;
      kin.add(up ? pk : -pk);
      if (K.thermal_solver) {
        float kj = gcol(P, G_KT, N, j);
        float w = up ? gcol(P, G_MRHO, N, j) : mrhoi;
        float dT = (thi - gcol(P, G_TH, N, j)) + (tli - gcol(P, G_TL, N, j));
        cond.add(w * 4.f * (ki * kj) / (ki + kj) * dT * g.GK);
      }
    }
    dkin = kin.value();
    double sr[6];
    for (int c = 0; c < 6; ++c) sr[c] = col(P, C_SR + c, N, i);
    if (K.thermal_solver) {
      double rho = col(P, C_RHO, N, i);
      double f = 1. / (rho * col(P, C_CPT, N, i));
      double dTdt = f * (cond.value() + col(P, C_QSRC, N, i) + col(P, C_QPL, N, i) * K.pl_work_heat_frac);
      colw(P, C_DTDT, N, i) = dTdt;
      double s = col(P, C_THEXP, N, i) * dTdt;
      for (int c = 0; c < 3; ++c) { sr[c] = sr[c] + s; colw(P, C_SR + c, N, i) = sr[c]; }
    }
    double t[6];
    for (int c = 0; c < 6; ++c) t[c] = col(P, C_TAU + c, N, i);
    dint = col(P, C_MRHO, N, i) *
           (t[0] * sr[0] + 2.0 * t[3] * sr[3] + 2.0 * t[4] * sr[4] + t[1] * sr[1] + 2.0 * t[5] * sr[5] + t[2] * sr[2]);
    colw(P, C_DKIN, N, i) = dkin;
    colw(P, C_DINT, N, i) = dint;
  }
  double r;
  r = block_reduce<0>(dkin, sh); if (threadIdx.x == 0) P.partials[S_DKIN * K.nblocks + blockIdx.x] = r;
  r = block_reduce<0>(dint, sh); if (threadIdx.x == 0) P.partials[S_DINT * K.nblocks + blockIdx.x] = r;
}

void launch_refresh_shadows(const DevPtrs& P, const DomainConst& K, int force, cudaStream_t s) {
  k_refresh_shadows<<<nblk(K.N, BLOCK), BLOCK, 0, s>>>(P, K, force);
  mark(s, "k_refresh_shadows");
}

void launch_step_mixed(const DevPtrs& P, const DomainConst& K, double* fscratch, int* iscratch, cudaStream_t s) {
  int nb = nblk(K.N, BLOCK);
  launch_step_head(P, K, fscratch, iscratch, s);
  launch_refresh_shadows(P, K, 0, s);
  k_accel_mx<<<nb, BLOCK, 0, s>>>(P, K);
  mark(s, "k_accel_mx");
  launch_bc(P, K, C_V, s);
  launch_contact_kick(P, K, s);
  launch_bc(P, K, C_V, s);
  k_density_drift_mx<<<nb, BLOCK, 0, s>>>(P, K);
  mark(s, "k_density_drift_mx");
  launch_bc(P, K, C_VN, s);
  float* rates = P.g + (size_t)G_RATES * K.N;
  k_rate_mx<<<nb, BLOCK, 0, s>>>(P, K, rates);
  mark(s, "k_rate_mx");
  k_stress_mx<<<nb, BLOCK, 0, s>>>(P, K, rates);
  mark(s, "k_stress_mx");
  k_energy_mx<<<nb, BLOCK, 0, s>>>(P, K);
  mark(s, "k_energy_mx");
  launch_step_tail(P, K, s);
}

}  // namespace wf
