// Mixed FP32/FP64 form of the kick-drift step on sm_103a.
//
// Same step, same reference semantics as the plain form (wf_step_fp64.cu);
// what changes is how the pair gathers compute and what they read:
//  * the FP32 gather data sits in float4 field-group columns (group q of
//    particle i at rc[q*N + i]), so a neighbour costs four 16-byte loads
//    (five when h, mass or Cs differ between the particles of a pair) that
//    coalesce across the warp's consecutive particles, instead of one scalar
//    load from each of ~20 separate columns;
//  * relative positions, velocities and temperatures come from float-float
//    pairs, (hi_i - hi_j) + (lo_i - lo_j), with FP32 instructions only (GB300
//    issues FP64 at 1/72 of its FP32 rate).  Temperature low halves are FP32,
//    which gives the FP32 rounding of the FP64 difference; position and
//    velocity low halves are bf16, which adds at most ~2^-33 |x - O| (O the
//    records' origin, the cell grid's centre) or ~2^-33 |v| to the difference
//    (the bound is in wf_device.cuh beside the record layout);
//  * kernel gradients, viscosity and pair terms in FP32, every per-particle
//    pair sum Kahan-compensated;
//  * FP64 stays in position/velocity/density/temperature integration, the
//    stress accumulation with its radial-return yield check and scale factor,
//    and all global reductions.
// Three gathers per step: acceleration; density (+ drift and second kick);
// rate tensors fused with the kinetic-energy and conduction sums, which use
// the same positions, velocities and the pressure of the updated density.
// Each walks a particle's row with one thread, or on small domains with
// 2-8 lanes whose partial sums are combined by warp shuffles.
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

__device__ __forceinline__ float4 ld4(const float4* p) { return __ldg(p); }

// One thread per particle: block b handles particles [b*B, (b+1)*B).
template <class Body>
__device__ __forceinline__ void run_rows(const DomainConst& K, Body body) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < K.N) body(i);
}

// Cubic-spline gradient factor GK (Functions.cpp:74-87, 3D) from r^2 and the
// pair smoothing length hh = (hi + hj) / 2.
__device__ __forceinline__ float grad_kernel_f(float r2, float hh, float* r_out) {
  float rinv = rsqrtf(r2);
  float r = r2 * rinv;
  float inv_h = 1.0f / hh;
  float q = r * inv_h;
  float ih2 = inv_h * inv_h;
  float C = INV_PI_F * ih2 * ih2 * inv_h;
  float w;
  if (q < 1.0f) w = -3.0f + 2.25f * q;
  else if (q < 2.0f) { float t = 2.0f - q; w = -0.75f * t * t * (hh * rinv); }
  else w = 0.0f;
  if (r2 == 0.0f) { w = -3.0f; r = 0.0f; }
  *r_out = r;
  return C * w;
}

// The same factor for a pair smoothing length hh = h that is uniform over the
// domain: 1/h and C come precomputed (the same FP32 operations on the host).
template <bool UNI>
__device__ __forceinline__ float grad_kernel(const DomainConst& K, float r2, float hh, float* r_out) {
  if (!UNI) return grad_kernel_f(r2, hh, r_out);
  float rinv = rsqrtf(r2);
  float r = r2 * rinv;
  float q = r * K.inv_h_f;
  float w;
  if (q < 1.0f) w = -3.0f + 2.25f * q;
  else if (q < 2.0f) { float t = 2.0f - q; w = -0.75f * t * t * (K.h_f * rinv); }
  else w = 0.0f;
  if (r2 == 0.0f) { w = -3.0f; r = 0.0f; }
  *r_out = r;
  return K.gk_c_f * w;
}

// Kernel-gradient correction of the locking sums (gradKernelCorr): the
// corrected gradient Mult(GK gradCorrM_i, x_ij) (InteractionAlt.cpp:114-132),
// with the particle's own matrix in FP32.
struct CorrM {
  float m[9];
};
__device__ __forceinline__ CorrM load_corr(const DevPtrs& P, size_t N, int i) {
  CorrM c;
  for (int k = 0; k < 9; ++k) c.m[k] = (float)col(P, C_GCM + k, N, i);
  return c;
}
__device__ __forceinline__ void corr_gk(const CorrM& c, float GK, float x0, float x1, float x2, float& g0, float& g1,
                                        float& g2) {
  g0 = GK * (c.m[0] * x0 + c.m[1] * x1 + c.m[2] * x2);
  g1 = GK * (c.m[3] * x0 + c.m[4] * x1 + c.m[5] * x2);
  g2 = GK * (c.m[6] * x0 + c.m[7] * x1 + c.m[8] * x2);
}

// ---------------------------------------------------------------- records
__global__ void k_refresh_records(DevPtrs P, DomainConst K, int force) {
  // After a search that reordered the particles (a filter-only search keeps
  // the order, and every step writes the records from the FP64 state).
  if (!force && !(P.st->do_search && P.st->search_full)) return;
  size_t N = K.N;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K.N; i += gridDim.x * blockDim.x) {
  bool solid = icol(P, I_KIND, N, i) == 0;
  double rho = col(P, C_RHO, N, i);
  double c2 = solid ? 1.0 / (rho * rho) : 0.0;
  float xh[3], xl[3], vh[3], vl[3], th, tl;
  for (int d = 0; d < 3; ++d) {
    ff_split(col(P, C_X + d, N, i) - K.rec_origin[d], xh[d], xl[d]);
    ff_split(col(P, C_V + d, N, i), vh[d], vl[d]);
  }
  ff_split(col(P, C_T, N, i), th, tl);
  float4* r = P.rc + i;
  // uniform-particle layout: Sigma/rho^2 xz, yz in the .w slots of the x and v groups
  float w_x = K.uni ? (float)(c2 * col(P, C_SIG + 4, N, i)) : (float)col(P, C_H, N, i);
  float w_v = K.uni ? (float)(c2 * col(P, C_SIG + 5, N, i)) : (float)rho;
  r[(size_t)RC_XH * N] = make_float4(xh[0], xh[1], xh[2], w_x);
  r[(size_t)RC_L * N] = lo_pack(xl, vl, solid ? (float)(col(P, C_MASS, N, i) / rho) : 0.f);
  r[(size_t)RC_VH * N] = make_float4(vh[0], vh[1], vh[2], w_v);
  r[(size_t)RC_S0 * N] = make_float4((float)(c2 * col(P, C_SIG, N, i)), (float)(c2 * col(P, C_SIG + 1, N, i)),
                         (float)(c2 * col(P, C_SIG + 2, N, i)), (float)(c2 * col(P, C_SIG + 3, N, i)));
  r[(size_t)RC_S1 * N] = make_float4((float)(c2 * col(P, C_SIG + 4, N, i)), (float)(c2 * col(P, C_SIG + 5, N, i)),
                         (float)col(P, C_MASS, N, i), (float)col(P, C_CS, N, i));
  r[(size_t)RC_MISC * N] = make_float4((float)col(P, C_ALPHA, N, i), (float)col(P, C_BETA, N, i), (float)col(P, C_KT, N, i), th);
  r[(size_t)RC_T2 * N] = make_float4(tl, 0.f, 0.f, 0.f);
  }
}

// ---------------------------------------------------------------- accel
// AVU: every solid particle has the same (alpha, beta), so the pair mean is
// the value itself and the gather reads neither particle's misc group.
// GC: kernel-gradient correction (temp_c = Mult(vc_i, S), InteractionAlt.cpp:166-170).
// Where a gather reads its neighbours' float4 groups: global memory through
// the row's indices, or a block's staged halo through the row's slots.
// A fetch splits into the row entry's reference (key) and the records it
// points at, so a gather can load entry k + dk's key before it consumes
// entry k's records: the index load then overlaps the record loads instead of
// adding a second memory latency to every iteration.
struct GlobalFetch {
  const float4* rc;
  const int* nb;  // P.nbr + i
  size_t N;
  __device__ __forceinline__ int key(int k) const { return nb_index(nb[(size_t)k * N]); }
  template <bool UNI = false>
  __device__ __forceinline__ int get(int j, float4& xh, float4& lo, float4& vh, float4& s0, float4& s1) const {
    const float4* rj = rc + j;
    xh = ld4(rj + (size_t)RC_XH * N); lo = ld4(rj + (size_t)RC_L * N); vh = ld4(rj + (size_t)RC_VH * N);
    s0 = ld4(rj + (size_t)RC_S0 * N);
    if (!UNI) s1 = ld4(rj + (size_t)RC_S1 * N);  // uniform layout: xz, yz ride in xh.w, vh.w
    return j;
  }
};
struct StagedFetch {
  const float4* sh;            // 5 groups of cap records in shared memory
  const unsigned short* slot;  // P.nslot + i
  size_t N;
  int cap;
  __device__ __forceinline__ int key(int k) const { return slot[(size_t)k * N]; }
  template <bool UNI = false>
  __device__ __forceinline__ int get(int q, float4& xh, float4& lo, float4& vh, float4& s0, float4& s1) const {
    xh = sh[q]; lo = sh[cap + q]; vh = sh[2 * cap + q]; s0 = sh[3 * cap + q]; s1 = sh[4 * cap + q];
    return -1;  // the global index is not known here: no misc or TI group (AVU and !TI only)
  }
};

// Pair sums of the acceleration of SPH particle i over row entries k0, k0 + dk, ...
// UNI: the uniform-particle layout (DomainConst::uni): h and Cs are the
// domain's constants, m_j = m_i, Sigma/rho^2 xz and yz come from the .w slots
// of the x and v groups, and rho_j = m_i / (m/rho)_j.
template <bool TI, bool AVU, bool GC, bool UNI, class Fetch>
__device__ __forceinline__ void accel_mx_sums(const DevPtrs& P, const DomainConst& K, int i, const Fetch& F, int k0,
                                              int dk, KSum& a0, KSum& a1, KSum& a2) {
  size_t N = K.N;
  const float4* ri = P.rc + i;
  float4 xh = ld4(ri + (size_t)RC_XH * N), lo = ld4(ri + (size_t)RC_L * N), vh = ld4(ri + (size_t)RC_VH * N);
  float xl[3], vl[3];
  lo_unpack(lo, xl, vl);
  float4 s0 = ld4(ri + (size_t)RC_S0 * N), s1;
  const float mass_i = UNI ? (float)col(P, C_MASS, N, i) : 0.f;
  if (UNI) s1 = make_float4(xh.w, vh.w, mass_i, K.cs_f);
  else s1 = ld4(ri + (size_t)RC_S1 * N);
  const float hi_ = UNI ? K.h_f : xh.w;
  const float rhoi = UNI ? (float)col(P, C_RHO, N, i) : vh.w;
  float4 mi = AVU ? make_float4(0.f, 0.f, 0.f, 0.f) : ld4(ri + (size_t)RC_MISC * N);
  float4 t0 = make_float4(0.f, 0.f, 0.f, 0.f), t1 = t0;
  if (TI) { t0 = ld4(ri + (size_t)RC_TI0 * N); t1 = ld4(ri + (size_t)RC_TI1 * N); }
  CorrM cm;
  if (GC) cm = load_corr(P, N, i);
  int len = P.row_len[i];
  int next = k0 < len ? F.key(k0) : 0;
  for (int k = k0; k < len; k += dk) {
    float4 jxh, jlo, jvh, js0, js1;
    int j = F.template get<UNI>(next, jxh, jlo, jvh, js0, js1);
    if (k + dk < len) next = F.key(k + dk);
    if (UNI) js1 = make_float4(jxh.w, jvh.w, mass_i, K.cs_f);
    const float4* rj = P.rc + j;
    float jxl[3], jvl[3];
    lo_unpack(jlo, jxl, jvl);
    float x0 = (xh.x - jxh.x) + (xl[0] - jxl[0]), x1 = (xh.y - jxh.y) + (xl[1] - jxl[1]), x2 = (xh.z - jxh.z) + (xl[2] - jxl[2]);
    float v0 = (vh.x - jvh.x) + (vl[0] - jvl[0]), v1 = (vh.y - jvh.y) + (vl[1] - jvl[1]), v2 = (vh.z - jvh.z) + (vl[2] - jvl[2]);
    float hh = UNI ? hi_ : 0.5f * (hi_ + jxh.w);
    float r2 = x0 * x0 + x1 * x1 + x2 * x2, r;
    float GK = grad_kernel<UNI>(K, r2, hh, &r);
    float Alpha, Beta;
    if (AVU) {
      Alpha = K.av_alpha; Beta = K.av_beta;
    } else {
      float4 jmi = ld4(rj + (size_t)RC_MISC * N);
      Alpha = 0.5f * (mi.x + jmi.x); Beta = 0.5f * (mi.y + jmi.y);
    }
    float PIs = 0.f;
    if (Alpha != 0.f || Beta != 0.f) {
      float dvx = v0 * x0 + v1 * x1 + v2 * x2;
      if (dvx < 0.f) {  // Monaghan viscosity (InteractionAlt.cpp:74-94)
        float MU = hh * dvx / (r * r + 0.01f * hh * hh);
        float Cij = 0.5f * (s1.w + js1.w);
        if (UNI)  // 1 / (0.5 (rho_i + rho_j)) with rho_j = m_i / (m/rho)_j
          PIs = (Alpha * Cij * MU + Beta * MU * MU) * (2.f * jlo.w) / (rhoi * jlo.w + mass_i);
        else
          PIs = (Alpha * Cij * MU + Beta * MU * MU) / (0.5f * (rhoi + jvh.w));
      }
    }
    float S0 = s0.x + js0.x + PIs, S1 = s0.y + js0.y + PIs, S2 = s0.z + js0.z + PIs;
    float S3 = s0.w + js0.w, S4 = s1.x + js1.x, S5 = s1.y + js1.y;
    if (TI) {  // tensile instability (InteractionAlt.cpp:102-109)
      // The reference adds the term when either end has TI > 0; TIR is zero
      // where TI is, so adding it for every pair with a finite factor (w0 > 0,
      // TIInitDist within the support) gives the same sums without reading
      // TI_j.
      float4 jt0 = ld4(rj + (size_t)RC_TI0 * N), jt1 = ld4(rj + (size_t)RC_TI1 * N);
      float q = r / hh, q0 = (t1.w + jt1.w) / (2.f * hh);
      float wq = q < 1.f ? 1.f - 1.5f * q * q + 0.75f * q * q * q : (q < 2.f ? 0.25f * (2.f - q) * (2.f - q) * (2.f - q) : 0.f);
      float w0 = q0 < 1.f ? 1.f - 1.5f * q0 * q0 + 0.75f * q0 * q0 * q0
                          : (q0 < 2.f ? 0.25f * (2.f - q0) * (2.f - q0) * (2.f - q0) : 0.f);
      if (w0 > 0.f) {
        float fb = wq / w0, fn = 0.5f * (t1.z + jt1.z);
        float f;
        if (fn == 4.f) { f = fb * fb; f = f * f; }  // the JSON driver's TIn (WeldForm.cpp:901)
        else f = powf(fb, fn);
        S0 += f * (t0.x + jt0.x); S1 += f * (t0.y + jt0.y); S2 += f * (t0.z + jt0.z);
        S3 += f * (t0.w + jt0.w); S4 += f * (t1.x + jt1.x); S5 += f * (t1.y + jt1.y);
      }
    }
    float g0 = GK * x0, g1 = GK * x1, g2 = GK * x2;
    if (GC) corr_gk(cm, GK, x0, x1, x2, g0, g1, g2);
    float mj = js1.z;
    a0.add(mj * (g0 * S0 + g1 * S3 + g2 * S4));
    a1.add(mj * (g0 * S3 + g1 * S1 + g2 * S5));
    a2.add(mj * (g0 * S4 + g1 * S5 + g2 * S2));
  }
}
template <bool TI, bool AVU, bool GC, bool UNI, class Fetch>
__device__ __forceinline__ void accel_mx(const DevPtrs& P, const DomainConst& K, int i, const Fetch& F) {
  size_t N = K.N;
  if (icol(P, I_KIND, N, i) != 0) {
    colw(P, C_A, N, i) = 0.0; colw(P, C_A + 1, N, i) = 0.0; colw(P, C_A + 2, N, i) = 0.0;
    return;
  }
  KSum a0, a1, a2;
  accel_mx_sums<TI, AVU, GC, UNI>(P, K, i, F, 0, 1, a0, a1, a2);
  colw(P, C_A, N, i) = a0.value(); colw(P, C_A + 1, N, i) = a1.value(); colw(P, C_A + 2, N, i) = a2.value();
}
template <bool TI, bool AVU, bool GC, bool UNI>
__global__ void __launch_bounds__(512) k_accel_mx(DevPtrs P, DomainConst K) {
  run_rows(K, [&](int i) { accel_mx<TI, AVU, GC, UNI>(P, K, i, GlobalFetch{P.rc, P.nbr + i, (size_t)K.N}); });
}

// L consecutive lanes share particle i = thread / L: lane s sums row entries
// s, s + L, s + 2L, ... with its own Kahan sums, and the L partial sums are
// combined in FP64 by a butterfly of __shfl_xor_sync (every lane ends with the
// same total; lane s == 0 writes it).  Each lane walks 1/L of the row, so a
// warp keeps loads of 32 / L particles' rows in flight with shorter dependent
// chains.  The result depends on L (summation order) but not on the block size.
template <bool TI, bool AVU, bool GC, bool UNI, int L>
__global__ void __launch_bounds__(512) k_accel_mx_lanes(DevPtrs P, DomainConst K) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = (int)(t / L), sub = (int)(t % L);
  const size_t N = K.N;
  const bool live = i < K.N;
  const bool sph = live && icol(P, I_KIND, N, i) == 0;
  KSum a0, a1, a2;
  if (sph) accel_mx_sums<TI, AVU, GC, UNI>(P, K, i, GlobalFetch{P.rc, P.nbr + i, N}, sub, L, a0, a1, a2);
  double v0 = a0.value(), v1 = a1.value(), v2 = a2.value();
  for (int off = 1; off < L; off <<= 1) {  // the whole warp takes part; L divides 32
    v0 += __shfl_xor_sync(0xffffffffu, v0, off);
    v1 += __shfl_xor_sync(0xffffffffu, v1, off);
    v2 += __shfl_xor_sync(0xffffffffu, v2, off);
  }
  if (live && sub == 0) {
    colw(P, C_A, N, i) = sph ? v0 : 0.0;
    colw(P, C_A + 1, N, i) = sph ? v1 : 0.0;
    colw(P, C_A + 2, N, i) = sph ? v2 : 0.0;
  }
}

// Staged acceleration gather (uniform viscosity constants, no tensile
// instability, no gradient correction): block b copies its halo's five groups
// into shared memory once, then two threads share each particle's row, which
// doubles the warps per SM that the shared-memory footprint allows.  The
// block's first STAGE_B threads sum the even row entries of its particles,
// the other STAGE_B the odd ones, so a warp's lanes still read the same entry
// k of consecutive particles (nearly consecutive slots, few bank conflicts);
// each half is a Kahan sum and the two are added in FP64.  A block whose halo
// exceeded the capacity (halo_len -1) reads global memory with the same split,
// so results do not depend on the capacity.
__global__ void __launch_bounds__(2 * STAGE_B) k_accel_mx_staged(DevPtrs P, DomainConst K) {
  extern __shared__ float4 sh_rec[];
  const int b = blockIdx.x, t = threadIdx.x, cap = K.stage_cap;
  const size_t N = K.N;
  const int H = P.halo_len[b];
  if (H > 0) {
    const int* hl = P.halo + (size_t)b * cap;
    for (int s = t; s < H; s += 2 * STAGE_B) {
      const float4* rj = P.rc + hl[s];
      sh_rec[s] = ld4(rj + (size_t)RC_XH * N);
      sh_rec[cap + s] = ld4(rj + (size_t)RC_L * N);
      sh_rec[2 * cap + s] = ld4(rj + (size_t)RC_VH * N);
      sh_rec[3 * cap + s] = ld4(rj + (size_t)RC_S0 * N);
      sh_rec[4 * cap + s] = ld4(rj + (size_t)RC_S1 * N);
    }
  }
  __syncthreads();
  const int p = t % STAGE_B, part = t / STAGE_B;
  const int i = b * STAGE_B + p;
  const bool sph = i < K.N && icol(P, I_KIND, N, i) == 0;
  KSum a0, a1, a2;
  if (sph) {
    if (H >= 0) accel_mx_sums<false, true, false, false>(P, K, i, StagedFetch{sh_rec, P.nslot + i, N, cap}, part, 2, a0, a1, a2);
    else accel_mx_sums<false, true, false, false>(P, K, i, GlobalFetch{P.rc, P.nbr + i, N}, part, 2, a0, a1, a2);
  }
  double v0 = a0.value(), v1 = a1.value(), v2 = a2.value();
  __syncthreads();  // halo records no longer read: the odd halves pass through shared memory
  double* ex = reinterpret_cast<double*>(sh_rec);  // 3 * STAGE_B doubles (stage_cap >= 64)
  if (part == 1) { ex[p] = v0; ex[STAGE_B + p] = v1; ex[2 * STAGE_B + p] = v2; }
  __syncthreads();
  if (part == 0 && i < K.N) {
    colw(P, C_A, N, i) = sph ? v0 + ex[p] : 0.0;
    colw(P, C_A + 1, N, i) = sph ? v1 + ex[STAGE_B + p] : 0.0;
    colw(P, C_A + 2, N, i) = sph ? v2 + ex[2 * STAGE_B + p] : 0.0;
  }
}

// ---------------------------------------------------------------- halo build
// After a search: for each block of STAGE_B consecutive particles, the
// distinct neighbour indices of its rows (a shared-memory hash set with
// bounded linear probing), compacted, sorted ascending (bitonic), stored as
// the block's halo, and each row entry's slot in it (binary search).  A block
// with more than stage_cap distinct neighbours is marked -1.  Gated on the
// search flag; a fixed grid strides over the blocks.
__global__ void __launch_bounds__(STAGE_B) k_halo_build(DevPtrs P, DomainConst K) {
  if (!P.st->do_search) return;
  __shared__ int tab[STAGE_HASH];
  __shared__ int keys[STAGE_CAP_MAX];
  __shared__ int s_cnt, s_over;
  __shared__ int s_wsum[STAGE_B / 32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const size_t N = K.N;
  const int cap = K.stage_cap;
  const int nsb = (K.N + STAGE_B - 1) / STAGE_B;
  constexpr int PER = STAGE_HASH / STAGE_B;
  for (int b = blockIdx.x; b < nsb; b += gridDim.x) {
    for (int s = t; s < STAGE_HASH; s += STAGE_B) tab[s] = -1;
    if (t == 0) { s_cnt = 0; s_over = 0; }
    __syncthreads();
    const int i = b * STAGE_B + t;
    const int len = i < K.N ? P.row_len[i] : 0;
    for (int k = 0; k < len; ++k) {
      int j = nb_index(P.nbr[(size_t)k * N + i]);
      unsigned h = ((unsigned)j * 2654435761u) >> 20;  // 12-bit hash
      int probe = 0;
      for (; probe < STAGE_HASH; ++probe) {
        int old = atomicCAS(&tab[h], -1, j);
        if (old == -1) { atomicAdd(&s_cnt, 1); break; }
        if (old == j) break;
        h = (h + 1) & (STAGE_HASH - 1);
      }
      if (probe == STAGE_HASH) s_over = 1;
    }
    __syncthreads();
    const int H = s_cnt;
    if (s_over || H > cap) {
      if (t == 0) P.halo_len[b] = -1;
      __syncthreads();
      continue;
    }
    // compaction: thread t owns hash slots [t * PER, (t + 1) * PER)
    int c = 0;
    for (int q = 0; q < PER; ++q) c += tab[t * PER + q] >= 0;
    int x = c;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_wsum[w] = x;
    __syncthreads();
    int pos = x - c;
    for (int q = 0; q < w; ++q) pos += s_wsum[q];
    for (int q = 0; q < PER; ++q) {
      int v = tab[t * PER + q];
      if (v >= 0) keys[pos++] = v;
    }
    int P2 = 1;
    while (P2 < H) P2 <<= 1;
    for (int q = H + t; q < P2; q += STAGE_B) keys[q] = 0x7fffffff;
    __syncthreads();
    for (int size = 2; size <= P2; size <<= 1)
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        for (int e = t; e < P2 / 2; e += STAGE_B) {
          int lo = 2 * e - (e & (stride - 1)), hi = lo + stride;
          bool asc = (lo & size) == 0;
          int a = keys[lo], bb = keys[hi];
          if ((a > bb) == asc) { keys[lo] = bb; keys[hi] = a; }
        }
        __syncthreads();
      }
    for (int q = t; q < H; q += STAGE_B) P.halo[(size_t)b * cap + q] = keys[q];
    if (t == 0) P.halo_len[b] = H;
    for (int k = 0; k < len; ++k) {
      int j = nb_index(P.nbr[(size_t)k * N + i]);
      int lo = 0, hi = H - 1;
      while (lo < hi) {
        int m = (lo + hi) >> 1;
        if (keys[m] < j) lo = m + 1; else hi = m;
      }
      P.nslot[(size_t)k * N + i] = (unsigned short)lo;
    }
    __syncthreads();
  }
}

void launch_halo_build(const DevPtrs& P, const DomainConst& K, cudaStream_t s) {
  int nsb = nblk(K.N, STAGE_B);
  k_halo_build<<<nsb < 152 * 4 ? nsb : 152 * 4, STAGE_B, 0, s>>>(P, K);
  mark(s, "k_halo_build");
}

int configure_staging(int cap) {
  size_t bytes = (size_t)5 * cap * sizeof(float4);
  return (int)cudaFuncSetAttribute(k_accel_mx_staged, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// ---------------------------------------------------------------- density + drift + kick
// GC: the locking sum with corrected gradients, m_j (rho_i / rho_j) v_ij . vc_i
// (InteractionAlt.cpp:589-605), which carries rho_i inside the sum.
// L lanes per particle (L = 1: one thread walks the row): lane `sub` sums
// entries sub, sub + L, ...; with L > 1 the lanes' compensated values are
// added in FP64 by a butterfly of warp shuffles (every thread of the warp
// takes part, so the caller runs this for out-of-range threads too, with
// live = false) and lane 0 finishes the particle.
// GC: the locking sum with corrected gradients, m_j (rho_i / rho_j) v_ij . vc_i
// (InteractionAlt.cpp:589-605), which carries rho_i inside the sum.
template <bool GC, bool UNI, int L>
__device__ __forceinline__ void density_drift_mx(const DevPtrs& P, const DomainConst& K, int i, int sub, bool live) {
  size_t N = K.N;
  double dt = P.st->deltat;
  double rhoi = live ? col(P, C_RHO, N, i) : 0.0;
  double dd = 0.0;
  bool solid = live && icol(P, I_KIND, N, i) == 0;
  const float4* ri = P.rc + i;
  float4 xh = live ? ld4(ri + (size_t)RC_XH * N) : make_float4(0.f, 0.f, 0.f, 0.f);
  if (solid) {
    float4 lo = ld4(ri + (size_t)RC_L * N), vh = ld4(ri + (size_t)RC_VH * N);
    float xl[3], vl[3];
    lo_unpack(lo, xl, vl);
    CorrM cm;
    if (GC) cm = load_corr(P, N, i);
    float rhoif = (float)rhoi;
    KSum s;
    int len = P.row_len[i];
    const int* nb = P.nbr + i;
    for (int k = sub; k < len; k += L) {
      int j = nb_index(nb[(size_t)k * N]);
      const float4* rj = P.rc + j;
      float4 jxh = ld4(rj + (size_t)RC_XH * N), jlo = ld4(rj + (size_t)RC_L * N), jvh = ld4(rj + (size_t)RC_VH * N);
      float jxl[3], jvl[3];
      lo_unpack(jlo, jxl, jvl);
      float x0 = (xh.x - jxh.x) + (xl[0] - jxl[0]), x1 = (xh.y - jxh.y) + (xl[1] - jxl[1]), x2 = (xh.z - jxh.z) + (xl[2] - jxl[2]);
      float v0 = (vh.x - jvh.x) + (vl[0] - jvl[0]), v1 = (vh.y - jvh.y) + (vl[1] - jvl[1]), v2 = (vh.z - jvh.z) + (vl[2] - jvl[2]);
      float r;
      float GK = grad_kernel<UNI>(K, x0 * x0 + x1 * x1 + x2 * x2, UNI ? K.h_f : 0.5f * (xh.w + jxh.w), &r);
      if (GC) {
        float g0, g1, g2;
        corr_gk(cm, GK, x0, x1, x2, g0, g1, g2);
        s.add(jlo.w * rhoif * (v0 * g0 + v1 * g1 + v2 * g2));  // m_j (rho_i / rho_j) = (m_j / rho_j) rho_i
      } else {
        s.add(jlo.w * (GK * (v0 * x0 + v1 * x1 + v2 * x2)));  // (m_j / rho_j) v_ij . (GK x_ij)
      }
    }
    dd = s.value();
  }
  if constexpr (L > 1)
    for (int off = 1; off < L; off <<= 1) dd += __shfl_xor_sync(0xffffffffu, dd, off);  // L divides 32
  if (!live || sub != 0) return;
  if (solid && !GC) dd *= rhoi;
  colw(P, C_DRHO, N, i) = dd;
  double rn = rhoi + dt * dd;
  colw(P, C_RHON, N, i) = rn;
  const double irn = 1.0 / rn;  // one FP64 division for m/rho and p/rho^2
  double mrn = solid ? col(P, C_MASS, N, i) * irn : 0.0;
  colw(P, C_MRHON, N, i) = mrn;
  float nxh[3], nxl[3], nvh[3], nvl[3];
  // GeneralAfter on the next-step velocity (SolverKickDrift.cpp:267) applied
  // here, records included, instead of in a BC pass after this kernel
  double vb[3];
  const bool bc = bc_velocity(P.tab, icol(P, I_ID, N, i), P.st->Time, vb);
  for (int d = 0; d < 3; ++d) {
    double v = col(P, C_V + d, N, i);
    double du = v * dt;
    colw(P, C_DISP + d, N, i) = col(P, C_DISP + d, N, i) + du;
    double xn = col(P, C_X + d, N, i) + du;
    double vn = bc ? vb[d] : (K.leapfrog ? v : v + col(P, C_A + d, N, i) * dt / 2.);
    if (bc) colw(P, C_A + d, N, i) = 0.0;
    colw(P, C_XN + d, N, i) = xn;
    colw(P, C_VN + d, N, i) = vn;
    ff_split(xn - K.rec_origin[d], nxh[d], nxl[d]);
    ff_split(vn, nvh[d], nvl[d]);
  }
  // Pressure of the updated density (EOS case 0, Functions.cpp:206-212) and the
  // temperature after this step's update (Thermal.cpp:727-734): both depend only
  // on this particle, so the fused rate/energy gather can read them.
  double cs = col(P, C_CS, N, i);
  double pn = col(P, C_P0, N, i) + (cs * cs) * (rn - col(P, C_RHO0, N, i));
  double Tn = col(P, C_T, N, i) + (K.thermal_solver ? dt * col(P, C_DTDT, N, i) : 0.0);
  float th, tl;
  ff_split(Tn, th, tl);
  float4* r = P.rn + i;
  r[(size_t)RN_XH * N] = make_float4(nxh[0], nxh[1], nxh[2], UNI ? K.h_f : xh.w);
  r[(size_t)RN_L * N] = lo_pack(nxl, nvl, (float)mrn);
  float pr2 = solid ? (float)(pn * irn * irn) : 0.f;
  r[(size_t)RN_VH * N] = make_float4(nvh[0], nvh[1], nvh[2], pr2);  // the rate gather reads p/rho^2 here
  r[(size_t)RN_E * N] = make_float4(pr2, ri[(size_t)RC_MISC * N].z, th, tl);
}
template <bool GC, bool UNI>
__global__ void __launch_bounds__(512, 3) k_density_drift_mx(DevPtrs P, DomainConst K) {
  run_rows(K, [&](int i) { density_drift_mx<GC, UNI, 1>(P, K, i, 0, true); });
}
template <bool GC, bool UNI, int L>
__global__ void __launch_bounds__(512) k_density_drift_mx_lanes(DevPtrs P, DomainConst K) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = (int)(t / L);
  density_drift_mx<GC, UNI, L>(P, K, i, (int)(t % L), i < K.N);
}

// ---------------------------------------------------------------- rates + energy + conduction
// Gather at x(n+1), v(n+1): strain/rotation rate sums (InteractionAlt.cpp:263-479),
// the kinetic-energy pair sum (Domain.cpp:1752-1808) and conduction (Thermal.cpp:53-219).
// GC: rates and conduction with corrected gradients (InteractionAlt.cpp:330-350,
// 425-450; Thermal.cpp:90-107), weights (float)(m_j / rho_j); the kinetic-energy
// pair term keeps the plain gradient, as the reference's.
// L lanes per particle (L = 1: one thread walks the row): lane `sub` sums
// entries sub, sub + L, ...; with L > 1 the lanes' compensated values are
// added in FP64 by a butterfly of warp shuffles (every thread of the warp
// takes part, so the caller runs this for out-of-range threads too, with
// live = false) and lane 0 writes the particle.
// KEEP: the particle's rates, kinetic-energy rate and conduction sum are
// handed to the caller in *ro instead of being stored (the fused rate-stress
// kernel; L = 1 only).
struct RateOut {
  float r[9];
  double dkin, cond;
};
template <bool THERMAL, bool GC, bool UNI, int L, bool KEEP = false>
__device__ __forceinline__ void rate_mx(const DevPtrs& P, const DomainConst& K, int i, int sub, bool live,
                                        RateOut* ro = nullptr) {
  static_assert(!KEEP || L == 1, "the rates are handed over by the thread that owns the row");
  size_t N = K.N;
  float out[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  double dkin = 0.0, cond = 0.0;
  const bool sph = live && icol(P, I_KIND, N, i) == 0;
  double md[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // L > 1: the lane's compensated values
  if (sph) {
    const float4* ri = P.rn + i;
    float4 xh = ld4(ri + (size_t)RN_XH * N), lo = ld4(ri + (size_t)RN_L * N), vh = ld4(ri + (size_t)RN_VH * N);
    float xl[3], vl[3];
    lo_unpack(lo, xl, vl);
    float4 e = THERMAL ? ld4(ri + (size_t)RN_E * N) : make_float4(vh.w, 0.f, 0.f, 0.f);
    CorrM cm;
    if (GC) cm = load_corr(P, N, i);
    KSum M[9];  // sum_j (m_j / rho_j) (-GK / 2) (v_i - v_j)_k (x_i - x_j)_l  (GC: gk_l for GK x_l)
    KSum kin, cnd;
    const float mass_i = (float)col(P, C_MASS, N, i);
    int len = P.row_len[i];
    const int* nb = P.nbr + i;
    for (int k = sub; k < len; k += L) {
      int ent = nb[(size_t)k * N];
      int j = nb_index(ent);
      const float4* rj = P.rn + j;
      float4 jxh = ld4(rj + (size_t)RN_XH * N), jlo = ld4(rj + (size_t)RN_L * N), jvh = ld4(rj + (size_t)RN_VH * N);
      float jxl[3], jvl[3];
      lo_unpack(jlo, jxl, jvl);
      // p/rho^2 rides in the velocity group; conduction needs the E group (k_T, T)
      float4 je = THERMAL ? ld4(rj + (size_t)RN_E * N) : make_float4(jvh.w, 0.f, 0.f, 0.f);
      float x0 = (xh.x - jxh.x) + (xl[0] - jxl[0]), x1 = (xh.y - jxh.y) + (xl[1] - jxl[1]), x2 = (xh.z - jxh.z) + (xl[2] - jxl[2]);
      float b0 = (vh.x - jvh.x) + (vl[0] - jvl[0]), b1 = (vh.y - jvh.y) + (vl[1] - jvl[1]), b2 = (vh.z - jvh.z) + (vl[2] - jvl[2]);
      float r;
      float GK = grad_kernel<UNI>(K, x0 * x0 + x1 * x1 + x2 * x2, UNI ? K.h_f : 0.5f * (xh.w + jxh.w), &r);
      float y0 = x0, y1 = x1, y2 = x2;
      float w = jlo.w * (-0.5f * GK);
      if (GC) {  // -1/2 (float)(m_j/rho_j) (v_ij (x) gk), gk = M_i GK x_ij
        corr_gk(cm, GK, x0, x1, x2, y0, y1, y2);
        w = jlo.w * -0.5f;
      }
      float wb0 = w * b0, wb1 = w * b1, wb2 = w * b2;
      M[0].add(wb0 * y0); M[1].add(wb0 * y1); M[2].add(wb0 * y2);
      M[3].add(wb1 * y0); M[4].add(wb1 * y1); M[5].add(wb1 * y2);
      M[6].add(wb2 * y0); M[7].add(wb2 * y1); M[8].add(wb2 * y2);
      bool up = nb_up(ent);  // original index of j larger than i's
      float dv = GK * (b0 * x0 + b1 * x1 + b2 * x2);
      // m_P2 of the pair: m_i when the pairs' masses agree, else the column
      float mP2 = K.m_pair ? mass_i : (float)col(P, C_MASS, N, up ? j : i);
      float pk = 0.5f * mP2 * (e.x + je.x) * dv;
      kin.add(up ? pk : -pk);
      if (THERMAL) {
        float wt = up ? jlo.w : lo.w;  // m_P2 / rho_P2 for both ends of the pair
        float dT = (e.z - je.z) + (e.w - je.w);
        // x.(GK x)/r^2 = GK; with the correction x.gk/r^2 (Thermal.cpp:90-107)
        float gr = GC ? (x0 * y0 + x1 * y1 + x2 * y2) / (x0 * x0 + x1 * x1 + x2 * x2) : GK;
        cnd.add(wt * 4.f * (e.y * je.y) / (e.y + je.y) * dT * gr);
      }
    }
    if constexpr (L == 1) {
      // The rate columns are FP32: each compensated sum is rounded to FP32 once
      // (s - c) and combined in FP32, which keeps the epilogue off the FP64 pipe.
      float m[9];
      for (int c = 0; c < 9; ++c) m[c] = M[c].s - M[c].c;
      out[0] = 2.0f * m[0]; out[1] = 2.0f * m[4]; out[2] = 2.0f * m[8];
      out[3] = m[1] + m[3]; out[4] = m[2] + m[6]; out[5] = m[5] + m[7];
      out[6] = m[1] - m[3]; out[7] = m[2] - m[6]; out[8] = m[5] - m[7];
    } else {
      for (int c = 0; c < 9; ++c) md[c] = M[c].value();
    }
    dkin = kin.value();
    cond = cnd.value();
  }
  if constexpr (L > 1) {
    for (int off = 1; off < L; off <<= 1) {  // L divides 32
      for (int c = 0; c < 9; ++c) md[c] += __shfl_xor_sync(0xffffffffu, md[c], off);
      dkin += __shfl_xor_sync(0xffffffffu, dkin, off);
      if (THERMAL) cond += __shfl_xor_sync(0xffffffffu, cond, off);
    }
    if (sph) {
      float m[9];
      for (int c = 0; c < 9; ++c) m[c] = (float)md[c];
      out[0] = 2.0f * m[0]; out[1] = 2.0f * m[4]; out[2] = 2.0f * m[8];
      out[3] = m[1] + m[3]; out[4] = m[2] + m[6]; out[5] = m[5] + m[7];
      out[6] = m[1] - m[3]; out[7] = m[2] - m[6]; out[8] = m[5] - m[7];
    }
  }
  if (!live || sub != 0) return;
  if constexpr (KEEP) {
    for (int c = 0; c < 9; ++c) ro->r[c] = out[c];
    ro->dkin = dkin;
    ro->cond = cond;
    return;
  }
  for (int c = 0; c < 9; ++c) P.rates[(size_t)c * N + i] = out[c];
  colw(P, C_DKIN, N, i) = dkin;
  colw(P, C_DINT, N, i) = cond;  // conduction sum, consumed by k_stress_mx
}
template <bool THERMAL, bool GC, bool UNI>
__global__ void __launch_bounds__(512) k_rate_mx(DevPtrs P, DomainConst K) {
  run_rows(K, [&](int i) { rate_mx<THERMAL, GC, UNI, 1>(P, K, i, 0, true); });
}
template <bool THERMAL, bool GC, bool UNI, int L>
__global__ void __launch_bounds__(512) k_rate_mx_lanes(DevPtrs P, DomainConst K) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = (int)(t / L);
  rate_mx<THERMAL, GC, UNI, L>(P, K, i, (int)(t % L), i < K.N);
}

// ---------------------------------------------------------------- elementwise update
// Stress state of the radial return.  The strain columns (Strain, Strain_pl,
// Strain_pl_incr) are not held here: the kernel streams them after the return,
// which keeps the kernel's register footprint small.
struct StressMx {
  double tau[6], sig[6];
  double pressure, pl_strain, delta_pl_strain, sigmay, Ep;
  float esr;
};

// Radial return with the Jaumann increment formed in FP32 and accumulated into
// the FP64 deviatoric stress; yield check, scale factor and plastic increment
// in FP64 (Particle.cpp:960-1067).  Returns the plastic increment.  The trial
// stress sqrt(3 J2) and the ratio sigma_y / sigma_trial are formed only when
// 3 J2 > sigma_y^2 (a particle inside the yield surface has scale factor 1 and
// no plastic step), so elastic particles skip the FP64 sqrt and divide.
__device__ __forceinline__ double stress_update_mx(StressMx& s, const float sr[6], const float rr[3], double rho,
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
    t6[c] = s.tau[c] + (double)(dtf * (twoG * dev + srt + rs));
  }
  float d01 = sr[0] - sr[1], d12 = sr[1] - sr[2], d20 = sr[2] - sr[0];
  s.esr = sqrtf(0.5f * (d01 * d01 + d12 * d12 + d20 * d20) + 3.0f * (sr[3] * sr[3] + sr[5] * sr[5] + sr[4] * sr[4]));
  double dep = 0.0;
  if (fail == 1) {
    double J2 = 0.5 * (t6[0] * t6[0] + 2.0 * t6[3] * t6[3] + 2.0 * t6[4] * t6[4] + t6[1] * t6[1] +
                       2.0 * t6[5] * t6[5] + t6[2] * t6[2]);
    double tJ2 = 3.0 * J2;
    double sig_trial = -1.0;  // sqrt(3 J2), formed on demand
    double sy = s.sigmay;
    if (!(sy > 0.0 && tJ2 <= sy * sy)) {
      sig_trial = sqrt(tJ2);
      double ratio = sy / sig_trial;
      double sc = (1.0 < ratio) ? 1.0 : ratio;  // std::min(ratio, 1.0)
      if (sc != 1.0)
        for (int c = 0; c < 6; ++c) t6[c] = sc * t6[c];
    }
    if (model == 1 && M) {
      if (s.pl_strain + M->eps0 > M->eps1) s.sigmay = (double)((float)M->K * powf((float)(s.pl_strain + M->eps0), (float)M->m));
      else s.sigmay = M->sy0;
    } else if (model == 2 && M) {
      float Th = (float)((T - M->T_t) / (M->T_m - M->T_t));
      float f = 1.0f;
      if (s.esr > (float)M->eps_0) f = 1.0f + (float)M->C * logf(s.esr / (float)M->eps_0);
      s.sigmay = (double)(((float)M->A + (float)M->B * powf((float)s.pl_strain, (float)M->n)) * f *
                          (1.0f - powf(Th, (float)M->jm)));
    }
    sy = s.sigmay;
    if (!(sy > 0.0 && tJ2 <= sy * sy)) {
      if (sig_trial < 0.0) sig_trial = sqrt(tJ2);
      if (sig_trial > sy) {
        if (s.Ep < 0) s.Ep = M ? M->E : 0.0;
        dep = (sig_trial - sy) / (3. * G + s.Ep);
        s.pl_strain += dep;
        s.delta_pl_strain = dep;
        if (model == 0) s.sigmay += dep * s.Ep;
      }
    }
  }
  for (int c = 0; c < 6; ++c) s.tau[c] = t6[c];
  for (int c = 0; c < 6; ++c) s.sig[c] = (c < 3 ? -s.pressure : 0.0) + t6[c];
  return dep;
}

// The per-particle update after the rate gather, with the block's partial
// sums.  FUSED: the rates, kinetic-energy rate and conduction sum come in ro
// from the same thread's gather (k_rate_stress_mx) rather than from the
// columns k_rate_mx stores; every thread of the block calls it (i >= N
// included) for the block reductions.
template <bool HEAT, bool THERMAL, bool FUSED>
__device__ __forceinline__ void stress_mx(const DevPtrs& P, const DomainConst& K, int i, const RateOut& ro) {
  __shared__ double sh[32];
  size_t N = K.N;
  double dt = P.st->deltat;
  double plw = 0.0, maxpl = 0.0, maxT = -1e300, minT = 1e300, dkin = 0.0, dint = 0.0;
  if (i < K.N) {
    for (int d = 0; d < 3; ++d) {
      colw(P, C_X + d, N, i) = col(P, C_XN + d, N, i);
      colw(P, C_V + d, N, i) = col(P, C_VN + d, N, i);
    }
    double rho = col(P, C_RHON, N, i);
    colw(P, C_RHO, N, i) = rho;
    colw(P, C_MRHO, N, i) = col(P, C_MRHON, N, i);
    const float4* rn = P.rn + i;
    float4* rc = P.rc + i;
    float4 nxh = rn[(size_t)RN_XH * N];
    rc[(size_t)RC_L * N] = rn[(size_t)RN_L * N];
    float4 nvh = rn[(size_t)RN_VH * N];
    // the current groups carry h and rho (the acceleration gather's viscosity),
    // or in the uniform-particle layout Sigma/rho^2 xz and yz (written below
    // for SPH particles, 0 for the rest)
    nxh.w = K.uni ? 0.f : nxh.w;
    nvh.w = K.uni ? 0.f : (float)rho;
    float4 ne = rn[(size_t)RN_E * N];
    float4 misc = rc[(size_t)RC_MISC * N];
    maxpl = col(P, C_PLS, N, i);
    const bool sph = icol(P, I_KIND, N, i) == 0;
    if constexpr (FUSED) {  // the columns k_rate_mx leaves behind (C_DINT: overwritten below for SPH particles)
      dkin = ro.dkin;
      colw(P, C_DKIN, N, i) = dkin;
      if (!sph) colw(P, C_DINT, N, i) = ro.cond;
    } else {
      dkin = col(P, C_DKIN, N, i);
    }
    if (sph) {
      float sr[6], rr[3];
      for (int c = 0; c < 6; ++c) sr[c] = FUSED ? ro.r[c] : P.rates[(size_t)c * N + i];
      for (int c = 0; c < 3; ++c) rr[c] = FUSED ? ro.r[6 + c] : P.rates[(size_t)(6 + c) * N + i];
      StressMx s;
      for (int c = 0; c < 6; ++c) s.tau[c] = col(P, C_TAU + c, N, i);
      s.pl_strain = col(P, C_PLS, N, i); s.delta_pl_strain = col(P, C_DPLS, N, i);
      s.sigmay = col(P, C_SY, N, i); s.Ep = col(P, C_EP, N, i);
      int mi = icol(P, I_MAT, N, i);
      const MaterialDev* Mt = (mi >= 0 && mi < P.tab->nmat) ? &P.tab->mat[mi] : nullptr;
      double T = col(P, C_T, N, i);
      double dep = stress_update_mx(s, sr, rr, rho, col(P, C_RHO0, N, i), col(P, C_CS, N, i), col(P, C_P0, N, i),
                                    col(P, C_G, N, i), T, icol(P, I_FAIL, N, i), icol(P, I_MODEL, N, i), Mt, dt);
      for (int c = 0; c < 6; ++c) {
        colw(P, C_TAU + c, N, i) = s.tau[c];
        colw(P, C_SIG + c, N, i) = s.sig[c];
        colw(P, C_EPS + c, N, i) = dt * (double)sr[c] + col(P, C_EPS + c, N, i);
      }
      // Strain_pl_incr = dep / sigma_y (sigma - tr-free part) and Strain_pl += it
      // (Particle.cpp:1040-1058); kept from the last plastic step otherwise.
      double epli[6];
      if (dep > 0.0) {
        double f = dep / s.sigmay;
        epli[0] = f * (s.sig[0] - 0.5 * (s.sig[1] + s.sig[2]));
        epli[1] = f * (s.sig[1] - 0.5 * (s.sig[0] + s.sig[2]));
        epli[2] = f * (s.sig[2] - 0.5 * (s.sig[0] + s.sig[1]));
        epli[3] = 1.5 * f * s.sig[3];
        epli[4] = 1.5 * f * s.sig[4];
        epli[5] = 1.5 * f * s.sig[5];
        for (int c = 0; c < 6; ++c) {
          colw(P, C_EPLI + c, N, i) = epli[c];
          colw(P, C_EPL + c, N, i) = col(P, C_EPL + c, N, i) + epli[c];
        }
      }
      double srd[6];
      for (int c = 0; c < 6; ++c) srd[c] = (double)sr[c];
      if (HEAT) {
        double q = col(P, C_QPL, N, i);
        if (s.delta_pl_strain > 0.0) {
          if (!(dep > 0.0))
            for (int c = 0; c < 6; ++c) epli[c] = col(P, C_EPLI + c, N, i);
          q = plastic_heat(s.sig, epli, dt);
        }
        colw(P, C_QPL, N, i) = q;
        colw(P, C_PSEN, N, i) = col(P, C_PSEN, N, i) + q * dt;
        plw = col(P, C_MASS, N, i) / rho * q;
      }
      if (THERMAL) {  // T(n+1) (already in the next record), then CalcTempInc's dTdt
        T += dt * col(P, C_DTDT, N, i);
        colw(P, C_T, N, i) = T;
        maxT = T; minT = T;
        double f = 1. / (rho * col(P, C_CPT, N, i));
        double qconv = conv_heat(P, N, i, rho, T);
        double dTdt = f * ((FUSED ? ro.cond : col(P, C_DINT, N, i)) + qconv + col(P, C_QSRC, N, i) + col(P, C_QPL, N, i) * K.pl_work_heat_frac);
        colw(P, C_DTDT, N, i) = dTdt;
        double st = col(P, C_THEXP, N, i) * dTdt;  // CalcThermalExpStrainRate
        for (int c = 0; c < 3; ++c) srd[c] = srd[c] + st;
      }
      for (int c = 0; c < 6; ++c) colw(P, C_SR + c, N, i) = srd[c];
      for (int c = 0; c < 3; ++c) colw(P, C_RR + c, N, i) = (double)rr[c];
      colw(P, C_P, N, i) = s.pressure; colw(P, C_PLS, N, i) = s.pl_strain; colw(P, C_DPLS, N, i) = s.delta_pl_strain;
      colw(P, C_SY, N, i) = s.sigmay; colw(P, C_EP, N, i) = s.Ep; colw(P, C_ESR, N, i) = (double)s.esr;
      maxpl = s.pl_strain;
      mark_yield(P, K, N, i, s.pl_strain);
      // CalcIntEnergyEqn (Particle.cpp:941-950)
      dint = col(P, C_MRHO, N, i) * (s.tau[0] * srd[0] + 2.0 * s.tau[3] * srd[3] + 2.0 * s.tau[4] * srd[4] +
                                     s.tau[1] * srd[1] + 2.0 * s.tau[5] * srd[5] + s.tau[2] * srd[2]);
      colw(P, C_DINT, N, i) = dint;
      float c2 = 1.0f / ((float)rho * (float)rho);
      rc[(size_t)RC_S0 * N] = make_float4(c2 * (float)s.sig[0], c2 * (float)s.sig[1], c2 * (float)s.sig[2], c2 * (float)s.sig[3]);
      if (K.uni) {
        nxh.w = c2 * (float)s.sig[4];
        nvh.w = c2 * (float)s.sig[5];
      } else {
        float4 s1o = rc[(size_t)RC_S1 * N];  // mass and Cs carried over
        rc[(size_t)RC_S1 * N] = make_float4(c2 * (float)s.sig[4], c2 * (float)s.sig[5], s1o.z, s1o.w);
      }
    }
    rc[(size_t)RC_XH * N] = nxh;
    rc[(size_t)RC_VH * N] = nvh;
    rc[(size_t)RC_MISC * N] = make_float4(misc.x, misc.y, misc.z, ne.z);
    rc[(size_t)RC_T2 * N] = make_float4(ne.w, 0.f, 0.f, 0.f);
  }
  double r;
  r = block_reduce<1>(maxpl, sh); if (threadIdx.x == 0) P.partials[S_MAXPL * K.nblocks + blockIdx.x] = r;
  r = block_reduce<0>(dkin, sh); if (threadIdx.x == 0) P.partials[S_DKIN * K.nblocks + blockIdx.x] = r;
  r = block_reduce<0>(dint, sh); if (threadIdx.x == 0) P.partials[S_DINT * K.nblocks + blockIdx.x] = r;
  if (HEAT) { r = block_reduce<0>(plw, sh); if (threadIdx.x == 0) P.partials[S_PLW * K.nblocks + blockIdx.x] = r; }
  if (THERMAL) {
    r = block_reduce<1>(maxT, sh); if (threadIdx.x == 0) P.partials[S_MAXT * K.nblocks + blockIdx.x] = r;
    r = block_reduce<2>(minT, sh); if (threadIdx.x == 0) P.partials[S_MINT * K.nblocks + blockIdx.x] = r;
  }
}
template <bool HEAT, bool THERMAL>
__global__ void __launch_bounds__(BLOCK, 3) k_stress_mx(DevPtrs P, DomainConst K) {
  stress_mx<HEAT, THERMAL, false>(P, K, blockIdx.x * blockDim.x + threadIdx.x, RateOut{});
}
// Rate gather and stress update in one launch (one thread per particle, the
// per-particle kernels' block size so the partial sums keep their layout):
// the nine rates stay in registers instead of a store and a reload.  Four
// blocks per SM cap it at the rate gather's own 64 registers (the update's
// FP64 state spills ~150 B to L1 once per particle): at 982,072 particles the
// step takes 1.267 against 1.313 ms with the two kernels; capped at 80
// registers (three blocks) the lost occupancy made it 3 % slower instead.  Within
// the launch the gather reads only the next-step records, the rows and the
// mass column, none of which the update writes, so the fusion has no
// ordering hazard, and the results are bit-identical to k_rate_mx followed
// by k_stress_mx.
template <bool THERMAL, bool GC, bool UNI, bool HEAT>
__global__ void __launch_bounds__(BLOCK, 4) k_rate_stress_mx(DevPtrs P, DomainConst K) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  RateOut ro;
  if (i < K.N) rate_mx<THERMAL, GC, UNI, 1, true>(P, K, i, 0, true, &ro);
  stress_mx<HEAT, THERMAL, true>(P, K, i, ro);
}

void launch_refresh_shadows(const DevPtrs& P, const DomainConst& K, int force, cudaStream_t s) {
  int b = nblk(K.N, BLOCK);
  k_refresh_records<<<b < 152 * 4 ? b : 152 * 4, BLOCK, 0, s>>>(P, K, force);
  mark(s, "k_refresh_records");
}

template <bool TI, bool AVU, bool GC, bool UNI>
static void launch_accel_mx_u(const DevPtrs& P, const DomainConst& K, int ng, int gb, cudaStream_t s) {
  // blocks for L lanes per particle: the grid covers L * N threads
  auto grid = [&](int L) { return (int)(((long long)K.N * L + gb - 1) / gb); };
  switch (K.glanes) {
    case 2: k_accel_mx_lanes<TI, AVU, GC, UNI, 2><<<grid(2), gb, 0, s>>>(P, K); break;
    case 4: k_accel_mx_lanes<TI, AVU, GC, UNI, 4><<<grid(4), gb, 0, s>>>(P, K); break;
    case 8: k_accel_mx_lanes<TI, AVU, GC, UNI, 8><<<grid(8), gb, 0, s>>>(P, K); break;
    default: k_accel_mx<TI, AVU, GC, UNI><<<ng, gb, 0, s>>>(P, K);
  }
}
// The density and rate gathers with the acceleration gather's lanes per particle.
template <bool GC, bool UNI>
static void launch_density_mx(const DevPtrs& P, const DomainConst& K, int ng, int gb, cudaStream_t s) {
  auto grid = [&](int L) { return (int)(((long long)K.N * L + gb - 1) / gb); };
  switch (K.glanes) {
    case 2: k_density_drift_mx_lanes<GC, UNI, 2><<<grid(2), gb, 0, s>>>(P, K); break;
    case 4: k_density_drift_mx_lanes<GC, UNI, 4><<<grid(4), gb, 0, s>>>(P, K); break;
    case 8: k_density_drift_mx_lanes<GC, UNI, 8><<<grid(8), gb, 0, s>>>(P, K); break;
    default: k_density_drift_mx<GC, UNI><<<ng, gb, 0, s>>>(P, K);
  }
}
template <bool THERMAL, bool GC, bool UNI>
static void launch_rate_mx(const DevPtrs& P, const DomainConst& K, int ng, int gb, cudaStream_t s) {
  auto grid = [&](int L) { return (int)(((long long)K.N * L + gb - 1) / gb); };
  switch (K.glanes) {
    case 2: k_rate_mx_lanes<THERMAL, GC, UNI, 2><<<grid(2), gb, 0, s>>>(P, K); break;
    case 4: k_rate_mx_lanes<THERMAL, GC, UNI, 4><<<grid(4), gb, 0, s>>>(P, K); break;
    case 8: k_rate_mx_lanes<THERMAL, GC, UNI, 8><<<grid(8), gb, 0, s>>>(P, K); break;
    default: k_rate_mx<THERMAL, GC, UNI><<<ng, gb, 0, s>>>(P, K);
  }
}
// The fused rate-stress kernel at the per-particle kernels' launch shape.
template <bool THERMAL, bool GC, bool UNI>
static void launch_rate_stress_mx(const DevPtrs& P, const DomainConst& K, cudaStream_t s) {
  if (K.pl_heating) k_rate_stress_mx<THERMAL, GC, UNI, true><<<K.nblocks, K.pblock, 0, s>>>(P, K);
  else k_rate_stress_mx<THERMAL, GC, UNI, false><<<K.nblocks, K.pblock, 0, s>>>(P, K);
}
template <bool TI, bool AVU>
static void launch_accel_mx(const DevPtrs& P, const DomainConst& K, int ng, int gb, cudaStream_t s) {
  if (K.gradcorr) {
    if (K.uni) launch_accel_mx_u<TI, AVU, true, true>(P, K, ng, gb, s);
    else launch_accel_mx_u<TI, AVU, true, false>(P, K, ng, gb, s);
  } else {
    if (K.uni) launch_accel_mx_u<TI, AVU, false, true>(P, K, ng, gb, s);
    else launch_accel_mx_u<TI, AVU, false, false>(P, K, ng, gb, s);
  }
}

void launch_step_mixed(const DevPtrs& P, const DomainConst& K, double* fscratch, int* iscratch, cudaStream_t s) {
  int nb = K.nblocks;
  int gb = (K.gblock == 64 || K.gblock == 128 || K.gblock == 512) ? K.gblock : 256;
  int ng = nblk(K.N, gb);
  launch_step_head(P, K, fscratch, iscratch, s);
  launch_tensile(P, K, s);
  const bool staged = K.stage_cap > 0 && P.halo && !K.ti && K.av_uniform && !K.gradcorr;
  if (staged) {
    k_accel_mx_staged<<<nblk(K.N, STAGE_B), 2 * STAGE_B, (size_t)5 * K.stage_cap * sizeof(float4), s>>>(P, K);
  } else if (K.ti) {
    if (K.av_uniform) launch_accel_mx<true, true>(P, K, ng, gb, s);
    else launch_accel_mx<true, false>(P, K, ng, gb, s);
  } else {
    if (K.av_uniform) launch_accel_mx<false, true>(P, K, ng, gb, s);
    else launch_accel_mx<false, false>(P, K, ng, gb, s);
  }
  mark(s, staged ? "k_accel_mx_staged" : "k_accel_mx");
  launch_bc(P, K, C_V, s);
  launch_contact_kick(P, K, s);
  if (K.leapfrog) launch_bc(P, K, C_V, s);  // kick-drift: applied by the kick kernel
  if (K.gradcorr) {
    if (K.uni) launch_density_mx<true, true>(P, K, ng, gb, s);
    else launch_density_mx<true, false>(P, K, ng, gb, s);
  } else {
    if (K.uni) launch_density_mx<false, true>(P, K, ng, gb, s);
    else launch_density_mx<false, false>(P, K, ng, gb, s);
  }
  mark(s, "k_density_drift_mx");  // the next-step BC applied by the density kernel
  // Fused rate-stress kernel: one lane per particle and no thermal solver
  // (the conduction terms would spill more at its 64-register budget; that
  // variant is not measured, so thermal workloads keep the two kernels).
  if (K.fuse_rs && K.glanes <= 1 && !K.thermal_solver) {
    if (K.gradcorr) { if (K.uni) launch_rate_stress_mx<false, true, true>(P, K, s); else launch_rate_stress_mx<false, true, false>(P, K, s); }
    else { if (K.uni) launch_rate_stress_mx<false, false, true>(P, K, s); else launch_rate_stress_mx<false, false, false>(P, K, s); }
    mark(s, "k_rate_stress_mx");
    launch_step_tail(P, K, s);
    return;
  }
  if (K.thermal_solver) {
    if (K.gradcorr) { if (K.uni) launch_rate_mx<true, true, true>(P, K, ng, gb, s); else launch_rate_mx<true, true, false>(P, K, ng, gb, s); }
    else { if (K.uni) launch_rate_mx<true, false, true>(P, K, ng, gb, s); else launch_rate_mx<true, false, false>(P, K, ng, gb, s); }
  } else {
    if (K.gradcorr) { if (K.uni) launch_rate_mx<false, true, true>(P, K, ng, gb, s); else launch_rate_mx<false, true, false>(P, K, ng, gb, s); }
    else { if (K.uni) launch_rate_mx<false, false, true>(P, K, ng, gb, s); else launch_rate_mx<false, false, false>(P, K, ng, gb, s); }
  }
  mark(s, "k_rate_mx");
  if (K.pl_heating) {
    if (K.thermal_solver) k_stress_mx<true, true><<<nb, K.pblock, 0, s>>>(P, K);
    else k_stress_mx<true, false><<<nb, K.pblock, 0, s>>>(P, K);
  } else {
    if (K.thermal_solver) k_stress_mx<false, true><<<nb, K.pblock, 0, s>>>(P, K);
    else k_stress_mx<false, false><<<nb, K.pblock, 0, s>>>(P, K);
  }
  mark(s, "k_stress_mx");
  launch_step_tail(P, K, s);
}

}  // namespace wf
