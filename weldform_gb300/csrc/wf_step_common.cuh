// Device helpers shared by the plain and mixed step kernels.
#pragma once
#include <cuda_bf16.h>

#include "wf_device.cuh"

namespace wf {

constexpr double WF_PI = 3.14159265358979323846;
constexpr double MIN_PS_FOR_NBSEARCH = 1.e-6;  // Source/Domain.cpp:28
constexpr int BLOCK = 256;                      // threads of the per-particle kernels

__device__ __forceinline__ double col(const DevPtrs& P, int c, size_t N, int i) { return P.f[(size_t)c * N + i]; }
__device__ __forceinline__ double& colw(const DevPtrs& P, int c, size_t N, int i) { return P.f[(size_t)c * N + i]; }
__device__ __forceinline__ int icol(const DevPtrs& P, int c, size_t N, int i) { return P.i[(size_t)c * N + i]; }

// Deterministic block reduction (fixed shuffle tree, then fixed order across
// warps) of one value per thread; the result is valid in thread 0.
template <int OP>  // 0 sum, 1 max, 2 min
__device__ __forceinline__ double block_reduce(double v, double* sh) {
  for (int off = 16; off > 0; off >>= 1) {
    double o = __shfl_down_sync(0xffffffffu, v, off);
    v = (OP == 0) ? v + o : (OP == 1 ? fmax(v, o) : fmin(v, o));
  }
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    int nw = blockDim.x >> 5;
    double r = sh[0];
    for (int k = 1; k < nw; ++k) r = (OP == 0) ? r + sh[k] : (OP == 1 ? fmax(r, sh[k]) : fmin(r, sh[k]));
    v = r;
  }
  return v;
}

// Float-float split of a double: hi = fl(v), lo = fl(v - hi).
__device__ __forceinline__ void ff_split(double v, float& hi, float& lo) {
  hi = __double2float_rn(v);
  lo = __double2float_rn(v - (double)hi);
}
__device__ __forceinline__ float* rc_f(const DevPtrs& P, size_t N, int i, int q) {
  return reinterpret_cast<float*>(P.rc + (size_t)q * N + i);
}
__device__ __forceinline__ float* rn_f(const DevPtrs& P, size_t N, int i, int q) {
  return reinterpret_cast<float*>(P.rn + (size_t)q * N + i);
}
// Low-half group: x = (xlo0, xlo1), y = (xlo2, vlo0), z = (vlo1, vlo2) as bf16
// pairs (first value in the low 16 bits), w = a float.  A bf16 is the upper
// half of an FP32, so unpacking is a shift or a mask.
__device__ __forceinline__ unsigned short bf16_bits(float f) { return __bfloat16_as_ushort(__float2bfloat16_rn(f)); }
__device__ __forceinline__ float bf16_pair(float a, float b) {
  return __uint_as_float((unsigned)bf16_bits(a) | ((unsigned)bf16_bits(b) << 16));
}
__device__ __forceinline__ float bf16_first(float p) { return __uint_as_float(__float_as_uint(p) << 16); }
__device__ __forceinline__ float bf16_second(float p) { return __uint_as_float(__float_as_uint(p) & 0xffff0000u); }
__device__ __forceinline__ float4 lo_pack(const float xl[3], const float vl[3], float w) {
  return make_float4(bf16_pair(xl[0], xl[1]), bf16_pair(xl[2], vl[0]), bf16_pair(vl[1], vl[2]), w);
}
__device__ __forceinline__ void lo_unpack(float4 g, float xl[3], float vl[3]) {
  xl[0] = bf16_first(g.x); xl[1] = bf16_second(g.x); xl[2] = bf16_first(g.y);
  vl[0] = bf16_second(g.y); vl[1] = bf16_first(g.z); vl[2] = bf16_second(g.z);
}
// v lo component d sits in 16-bit half 3 + d of the group.
__device__ __forceinline__ unsigned short* lo_v_half(float4* group, int d) {
  return reinterpret_cast<unsigned short*>(group) + 3 + d;
}

// Velocity component d of particle i into the current (next) float4 groups.
__device__ __forceinline__ void rec_set_v(const DevPtrs& P, size_t N, int i, int d, double v, bool next) {
  float h, l;
  ff_split(v, h, l);
  if (next) { rn_f(P, N, i, RN_VH)[d] = h; *lo_v_half(P.rn + (size_t)RN_L * N + i, d) = bf16_bits(l); }
  else { rc_f(P, N, i, RC_VH)[d] = h; *lo_v_half(P.rc + (size_t)RC_L * N + i, d) = bf16_bits(l); }
}

// The current velocity record of particle i from its three FP64 components
// (the .w field and the x lo halves carried over).
__device__ __forceinline__ void rec_set_v3(const DevPtrs& P, size_t N, int i, const double v[3]) {
  float4* r = P.rc + i;
  float4 h = r[(size_t)RC_VH * N];
  float l[3];
  ff_split(v[0], h.x, l[0]);
  ff_split(v[1], h.y, l[1]);
  ff_split(v[2], h.z, l[2]);
  r[(size_t)RC_VH * N] = h;
  for (int d = 0; d < 3; ++d) *lo_v_half(r + (size_t)RC_L * N, d) = bf16_bits(l[d]);
}

// Batched domain: flag the particle's specimen as yielding once its plastic
// strain passes the rebuild threshold (Domain.cpp:28), the per-specimen form of
// the max-plastic-strain test of the rebuild schedule.
__device__ __forceinline__ void mark_yield(const DevPtrs& P, const DomainConst& K, size_t N, int i, double pl) {
  if (K.nspec > 0 && pl > MIN_PS_FOR_NBSEARCH) {
    SpecState* sp = P.sp + icol(P, I_SPEC, N, i);
    if (!sp->yielded_next) sp->yielded_next = 1;
  }
}

// Amplitude lookup (SPH::amplitude::getValAtTime, Source/Domain.h:69-89).
__device__ __forceinline__ double amp_value(const DomainTables* T, int amp_id, double t, bool* found) {
  for (int k = 0; k < T->namp; ++k) {
    if (T->amp[k].id != amp_id) continue;
    *found = true;
    const double* tt = T->amp_t + T->amp[k].offset;
    const double* vv = T->amp_v + T->amp[k].offset;
    int i = T->amp[k].n - 1;
    bool end = false;
    while (!end) { i--; if (i == 0 || t > tt[i]) end = true; }
    return vv[i] + (vv[i + 1] - vv[i]) / (tt[i + 1] - tt[i]) * (t - tt[i]);
  }
  return 0.0;
}

// The velocity the BCs of zone id impose at time t (GeneralAfter,
// WeldForm.cpp:51-120): each of the zone's BCs in the order added, a later one
// overriding an earlier; an amplitude BC applies only where its table covers
// t.  False when none applies.  k_bc applies this to its list of BC
// particles; the kick and drift kernels apply it to their own particle in
// place of the BC passes that would follow them.
__device__ __forceinline__ bool bc_velocity(const DomainTables* T, int id, double t, double v[3]) {
  int lo, hi;
  bc_range(T, id, lo, hi);
  bool hit = false;
  for (int r = lo; r < hi; ++r) {
    const BCDev& b = T->bc[T->bc_order[r]];
    if (b.value_type == 0) {
      hit = true;
      for (int d = 0; d < 3; ++d) v[d] = b.value[d];
    } else {
      bool found = false;
      double val = b.amp_factor * amp_value(T, b.amp_id, t, &found);
      if (found) {
        hit = true;
        for (int d = 0; d < 3; ++d) v[d] = val * b.value[d];
      }
    }
  }
  return hit;
}

// CalcConvHeat (Thermal.cpp:339-389, 3D; Fraser Eq. 3-121): a particle with
// Thermal_BC == TH_BC_CONVECTION exchanges heat with the ambient temperature
// T_inf through its contact area dS^2 = (m / rho)^(2/3):
// q_conv = rho h_conv dS^2 (T_inf - T) / m, at the step's updated density and
// temperature.  Other particles keep their q_conv (0 from the constructor).
__device__ __forceinline__ double conv_heat(const DevPtrs& P, size_t N, int i, double rho, double T) {
  if (P.i[(size_t)I_THBC * N + i] != 1) return col(P, C_QCONV, N, i);
  double m = col(P, C_MASS, N, i);
  double dS2 = pow(m / rho, 2.0 / 3.0);
  double q = rho * col(P, C_HCONV, N, i) * dS2 * (col(P, C_TINF, N, i) - T) / m;
  colw(P, C_QCONV, N, i) = q;
  return q;
}

// Johnson-Cook flow stress (Source/Material.cpp:6-25).
__device__ __forceinline__ double jc_yield(const MaterialDev& M, double strain, double strain_rate, double temp) {
  double T_h = (temp - M.T_t) / (M.T_m - M.T_t);
  double f = 1.0;
  if (strain_rate > M.eps_0) f = (1.0 + M.C * log(strain_rate / M.eps_0));
  return (M.A + M.B * pow(strain, M.n)) * f * (1.0 - pow(T_h, M.jm));
}
// Hollomon flow stress with plateau (Source/Material.cpp:59-64).
__device__ __forceinline__ double hollomon_yield(const MaterialDev& M, double strain) {
  if (strain + M.eps0 > M.eps1) return M.K * pow(strain + M.eps0, M.m);
  return M.sy0;
}

// Cubic-spline kernel W(q) (Functions.cpp:25-36, 3D) without its constant
// 1/(pi h^3): the tensile-instability term only uses ratios of W.
__device__ __forceinline__ double kernel_shape(double q) {
  if (q < 1.0) return 1.0 - (3.0 / 2.0) * q * q + (3.0 / 4.0) * q * q * q;
  else if (q < 2.0) return (1.0 / 4.0) * (2.0 - q) * (2.0 - q) * (2.0 - q);
  return 0.0;
}

// Symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations (a published
// method; the reference calls GSL's gsl_eigen_symmv through Rotation,
// Functions.cpp:381-395).  s: xx yy zz xy xz yz.  Returns the eigenvalues in
// L and the eigenvectors as columns of V.  The sweep count is bounded.
__device__ __forceinline__ void eig_sym3(const double s[6], double L[3], double V[3][3]) {
  double a[3][3] = {{s[0], s[3], s[4]}, {s[3], s[1], s[5]}, {s[4], s[5], s[2]}};
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) V[r][c] = (r == c) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 50; ++sweep) {
    double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
    double diag = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
    if (off == 0.0 || off <= 1e-36 * diag) break;
    for (int e = 0; e < 3; ++e) {
      int p = e == 2 ? 1 : 0, q = e == 0 ? 1 : 2;
      if (a[p][q] == 0.0) continue;
      double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
      double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
      double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
      for (int k = 0; k < 3; ++k) {
        double akp = a[k][p], akq = a[k][q];
        a[k][p] = c * akp - sn * akq;
        a[k][q] = sn * akp + c * akq;
      }
      for (int k = 0; k < 3; ++k) {
        double apk = a[p][k], aqk = a[q][k];
        a[p][k] = c * apk - sn * aqk;
        a[q][k] = sn * apk + c * aqk;
      }
      for (int k = 0; k < 3; ++k) {
        double vkp = V[k][p], vkq = V[k][q];
        V[k][p] = c * vkp - sn * vkq;
        V[k][q] = sn * vkp + c * vkq;
      }
    }
  }
  for (int k = 0; k < 3; ++k) L[k] = a[k][k];
}

// The same cyclic Jacobi iteration in FP32, for the mixed form, whose
// tensile-instability stress enters the FP32 pair terms: converged to FP32
// resolution (off-diagonal squares below 1e-14 of the diagonal's).  A rotation
// angle beyond FP32 range takes t = 1 / (2 theta).
__device__ __forceinline__ void eig_sym3f(const float s[6], float L[3], float V[3][3]) {
  float a[3][3] = {{s[0], s[3], s[4]}, {s[3], s[1], s[5]}, {s[4], s[5], s[2]}};
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) V[r][c] = (r == c) ? 1.0f : 0.0f;
  for (int sweep = 0; sweep < 20; ++sweep) {
    float off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
    float diag = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
    if (off == 0.0f || off <= 1e-14f * diag) break;
    for (int e = 0; e < 3; ++e) {
      int p = e == 2 ? 1 : 0, q = e == 0 ? 1 : 2;
      if (a[p][q] == 0.0f) continue;
      float theta = (a[q][q] - a[p][p]) / (2.0f * a[p][q]);
      float t = fabsf(theta) > 1e15f ? 0.5f / theta
                                      : (theta >= 0.0f ? 1.0f : -1.0f) / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
      float c = rsqrtf(t * t + 1.0f), sn = t * c;
      for (int k = 0; k < 3; ++k) {
        float akp = a[k][p], akq = a[k][q];
        a[k][p] = c * akp - sn * akq;
        a[k][q] = sn * akp + c * akq;
      }
      for (int k = 0; k < 3; ++k) {
        float apk = a[p][k], aqk = a[q][k];
        a[p][k] = c * apk - sn * aqk;
        a[q][k] = sn * apk + c * aqk;
      }
      for (int k = 0; k < 3; ++k) {
        float vkp = V[k][p], vkq = V[k][q];
        V[k][p] = c * vkp - sn * vkq;
        V[k][q] = sn * vkp + c * vkq;
      }
    }
  }
  for (int k = 0; k < 3; ++k) L[k] = a[k][k];
}

// Radial-return constitutive update of one particle, Particle::CalcStressStrain
// (Source/Particle.cpp:960-1067), on symmetric storage (xx yy zz xy xz yz).
// sr: strain rate (6), rr: rotation rate (xy xz yz of the antisymmetric part).
// Returns dep (plastic strain increment).
struct StressIO {
  double tau[6], sig[6], eps[6], epl[6], epli[6];
  double pressure, pl_strain, delta_pl_strain, sigmay, Ep, esr;
  double sc = 1.0, sy_new = 0.0;  // branch record: scale factor and the step's flow stress
};
__device__ __forceinline__ double stress_update(StressIO& s, const double sr[6], const double rr[3], double rho,
                                                double rho0, double Cs, double P0, double G, double T, int fail,
                                                int model, const MaterialDev* M, double dt) {
  s.pressure = P0 + (Cs * Cs) * (rho - rho0);  // EOS case 0, Functions.cpp:206-212
  // Full matrices: S (symmetric tau), W (antisymmetric rotation rate).
  double S[3][3] = {{s.tau[0], s.tau[3], s.tau[4]}, {s.tau[3], s.tau[1], s.tau[5]}, {s.tau[4], s.tau[5], s.tau[2]}};
  double W[3][3] = {{0.0, rr[0], rr[1]}, {-rr[0], 0.0, rr[2]}, {-rr[1], -rr[2], 0.0}};
  // SRT = S W^T, RS = W S; entries summed k = 2, 1, 0 (matvec.h Mult order).
  const int ui[6] = {0, 1, 2, 0, 0, 1}, uj[6] = {0, 1, 2, 1, 2, 2};
  double tr = sr[0] + sr[1] + sr[2];
  double s3 = 1.0 / 3.0 * tr;
  double twoG = 2.0 * G;
  double t6[6];
  for (int c = 0; c < 6; ++c) {
    int a = ui[c], b = uj[c];
    double srt = S[a][2] * W[b][2] + S[a][1] * W[b][1] + S[a][0] * W[b][0];
    double rs = W[a][2] * S[2][b] + W[a][1] * S[1][b] + W[a][0] * S[0][b];
    double dev = sr[c] - (c < 3 ? s3 : 0.0);
    t6[c] = dt * (twoG * dev + srt + rs) + s.tau[c];
  }
  double d01 = sr[0] - sr[1], d12 = sr[1] - sr[2], d20 = sr[2] - sr[0];
  s.esr = sqrt(0.5 * (d01 * d01 + d12 * d12 + d20 * d20) + 3.0 * (sr[3] * sr[3] + sr[5] * sr[5] + sr[4] * sr[4]));
  double dep = 0.0;
  if (fail == 1) {
    double J2 = 0.5 * (t6[0] * t6[0] + 2.0 * t6[3] * t6[3] + 2.0 * t6[4] * t6[4] + t6[1] * t6[1] +
                       2.0 * t6[5] * t6[5] + t6[2] * t6[2]);
    double sig_trial = sqrt(3.0 * J2);
    double ratio = s.sigmay / sig_trial;
    double sc = (1.0 < ratio) ? 1.0 : ratio;  // std::min(ratio, 1.0)
    for (int c = 0; c < 6; ++c) t6[c] = sc * t6[c];
    if (model == 1 && M) s.sigmay = hollomon_yield(*M, s.pl_strain);
    else if (model == 2 && M) s.sigmay = jc_yield(*M, s.pl_strain, s.esr, T);
    s.sc = sc;
    s.sy_new = s.sigmay;
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
  for (int c = 0; c < 6; ++c) s.eps[c] = dt * sr[c] + s.eps[c];
  return dep;
}

// Plastic work heat source (Particle::CalcPlasticWorkHeat, Particle.cpp:922-939):
// q = Sigma : (Strain_pl_incr / dt) with the off-diagonal pairs doubled.
__device__ __forceinline__ double plastic_heat(const double sig[6], const double epli[6], double dt) {
  double f = 1. / dt;
  return sig[0] * (f * epli[0]) + 2.0 * sig[3] * (f * epli[3]) + 2.0 * sig[4] * (f * epli[4]) + sig[1] * (f * epli[1]) +
         2.0 * sig[5] * (f * epli[5]) + sig[2] * (f * epli[2]);
}

}  // namespace wf
