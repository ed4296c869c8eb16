// ============================================================================
// WeldForm kick-drift SPH solid step — CPU ORACLE (test infrastructure only).
//
// This file is the checker, not the product.  It restates, from the reference
// sources, the algorithms of the kick-drift solid path in plain C++ so that
// the GB300 library can be compared against it on identical inputs.  Only the
// test suite, the smoke check and the CPU-baseline leg of the benchmark load
// it.  Every routine cites the reference file:line it follows (paths relative
// to the WeldForm source tree).
//
// PARITY STATUS.  The reference cannot be compiled here (it needs blitz++,
// GSL and HDF5, none of which is present), so its physics has no golden
// vectors: the restated physics is "parity unpinned".  The particle generator
// and neighbour search ARE pinned: tests/golden holds the neighbour table the
// reference printed for particle 2000 of its CompressionVel example
// (Docs/reduction.txt:28-37), which this oracle reproduces.
//
// Two execution modes share the per-pair and per-particle arithmetic:
//   mode 0 "canonical"  — per-particle gather over a CSR whose rows are in the
//       canonical order (j > i ascending, then j < i ascending).  Deterministic
//       for any thread count; this is the parity reference.
//   mode 1 "reference"  — the reference's own structure: linked-list cell
//       search with OpenMP dynamic schedule over x-slabs into per-thread pair
//       lists (Neighbour.cpp:346-477), pair loops writing per-pair results,
//       then the Nishimura gather in insertion order (InteractionAlt.cpp).
//       This is the timed CPU baseline.
//
// Arithmetic follows the reference's evaluation order; build with
// -ffp-contract=off so no multiply-add is fused.
// ============================================================================
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#include <chrono>
#ifdef _OPENMP
#include <omp.h>
#endif

#define WF_OK               0
#define WF_ERR_ARG          1
#define WF_ERR_NAN          3
#define WF_ERR_NBR_OVERFLOW 4
#define WF_ERR_STATE        6
#define WF_ERR_UNSUPPORTED  8

namespace {

thread_local std::string g_err;
int set_err(int code, const std::string& msg) { g_err = msg; return code; }

const double PI = 3.14159265358979323846;  // M_PI
const double MIN_PS_FOR_NBSEARCH = 1.e-6;  // Domain.cpp:28
const int MAX_NB_PER_PART = 100;           // Domain.h:49

struct V3 { double c[3]; };
inline V3 v3(double a, double b, double c) { V3 r; r.c[0] = a; r.c[1] = b; r.c[2] = c; return r; }
inline V3 sub(const V3& a, const V3& b) { return v3(a.c[0] - b.c[0], a.c[1] - b.c[1], a.c[2] - b.c[2]); }
inline V3 add(const V3& a, const V3& b) { return v3(a.c[0] + b.c[0], a.c[1] + b.c[1], a.c[2] + b.c[2]); }
inline V3 scl(double s, const V3& a) { return v3(s * a.c[0], s * a.c[1], s * a.c[2]); }
// blitz::dot / norm on TinyVector<double,3>: left-to-right sum (blitz is not
// available here, so its exact association is unpinned).
inline double dot(const V3& a, const V3& b) { return a.c[0] * b.c[0] + a.c[1] * b.c[1] + a.c[2] * b.c[2]; }
inline double norm(const V3& a) { return std::sqrt(dot(a, a)); }
inline V3 cross(const V3& a, const V3& b) {
  return v3(a.c[1] * b.c[2] - a.c[2] * b.c[1], a.c[2] * b.c[0] - a.c[0] * b.c[2], a.c[0] * b.c[1] - a.c[1] * b.c[0]);
}
// 3x3 matrices stored row-major, 9 doubles (blitz TinyMatrix<double,3,3>).
struct M3 { double m[9]; };
inline double& at(M3& A, int i, int j) { return A.m[3 * i + j]; }
inline double at(const M3& A, int i, int j) { return A.m[3 * i + j]; }
inline M3 zero3() { M3 z; for (int k = 0; k < 9; ++k) z.m[k] = 0.0; return z; }
inline double I3(int i, int j) { return i == j ? 1.0 : 0.0; }
// matvec.h:829-834 Mult(Vec,Mat,Vec): B(c) = A0*M(0,c) + A1*M(1,c) + A2*M(2,c)
inline V3 vecmat(const V3& A, const M3& M) {
  V3 B;
  for (int c = 0; c < 3; ++c) B.c[c] = A.c[0] * at(M, 0, c) + A.c[1] * at(M, 1, c) + A.c[2] * at(M, 2, c);
  return B;
}
// matvec.h:845-851 Mult(Mat,Mat,Mat): every entry sums k = 2, 1, 0 in that order.
inline M3 matmul(const M3& A, const M3& B) {
  M3 C;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      at(C, i, j) = at(A, i, 2) * at(B, 2, j) + at(A, i, 1) * at(B, 1, j) + at(A, i, 0) * at(B, 0, j);
  return C;
}
inline M3 trans(const M3& A) { M3 T; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) at(T, i, j) = at(A, j, i); return T; }

// Functions.cpp:74-87 GradKernel, cubic spline (KernelType 0).
inline double grad_kernel(int dim, double q, double h) {
  double C = (dim == 2) ? 10.0 / (7.0 * h * h * h * PI) : 1.0 / (h * h * h * h * PI);
  if (q == 0.0) return C / h * (-3.0 + (9.0 / 2.0) * q);
  else if (q < 1.0) return C / (q * h) * (-3.0 * q + (9.0 / 4.0) * q * q);
  else if (q < 2.0) return C / (q * h) * ((-3.0 / 4.0) * (2.0 - q) * (2.0 - q));
  return 0.0;
}
// Functions.cpp:25-36 Kernel, cubic spline (KernelType 0).
inline double kernel_w(int dim, double q, double h) {
  double C = (dim == 2) ? 10.0 / (7.0 * h * h * PI) : 1.0 / (h * h * h * PI);
  if (q < 1.0) return C * (1.0 - (3.0 / 2.0) * q * q + (3.0 / 4.0) * q * q * q);
  else if (q < 2.0) return C * ((1.0 / 4.0) * (2.0 - q) * (2.0 - q) * (2.0 - q));
  return 0.0;
}
// Symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations, standing in
// for gsl_eigen_symmv (matvec.h:776-803, GSL not available here): eigenvalues
// L (ascending, as Rotation's SortAsc) and eigenvectors as the columns of V.
// Functions of the spectrum that do not depend on the eigenvector basis (the
// tensile-instability stress below) agree with any backward-stable solver to
// rounding.
inline void eig_sym3(const M3& M, double L[3], M3& V) {
  double a[3][3];
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) a[i][j] = 0.5 * (at(M, i, j) + at(M, j, i));
  double v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int sweep = 0; sweep < 50; ++sweep) {
    double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
    double diag = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
    if (off <= 1e-36 * diag || off == 0.0) break;
    const int pq[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (auto& e : pq) {
      int p = e[0], q = e[1];
      if (a[p][q] == 0.0) continue;
      double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
      double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
      double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
      for (int k = 0; k < 3; ++k) {  // A <- A J (columns p, q)
        double akp = a[k][p], akq = a[k][q];
        a[k][p] = c * akp - sn * akq;
        a[k][q] = sn * akp + c * akq;
      }
      for (int k = 0; k < 3; ++k) {  // A <- J^T A (rows p, q)
        double apk = a[p][k], aqk = a[q][k];
        a[p][k] = c * apk - sn * aqk;
        a[q][k] = sn * apk + c * aqk;
      }
      for (int k = 0; k < 3; ++k) {
        double vkp = v[k][p], vkq = v[k][q];
        v[k][p] = c * vkp - sn * vkq;
        v[k][q] = sn * vkp + c * vkq;
      }
    }
  }
  int ord[3] = {0, 1, 2};
  std::sort(ord, ord + 3, [&](int x, int y) { return a[x][x] < a[y][y]; });
  for (int k = 0; k < 3; ++k) {
    L[k] = a[ord[k]][ord[k]];
    for (int r = 0; r < 3; ++r) at(V, r, k) = v[r][ord[k]];
  }
}

// Functions.cpp:206-212 EOS case 0.
inline double eos0(double Cs, double P0, double rho, double rho0) { return P0 + (Cs * Cs) * (rho - rho0); }

struct Material {
  int model = 0;
  double E = 0, nu = 0;
  // Hollomon (Material.cpp:48-72)
  double K = 0, m = 0, eps0 = 0, eps1 = 0, sy0 = 0;
  // Johnson-Cook (Material.h:117-151, Material.cpp:6-46)
  double A = 0, B = 0, C = 0, n = 0, jm = 0, eps_0 = 0, T_m = 0, T_t = 0;
  // Material.cpp:6-25 JohnsonCook::CalcYieldStress
  double jc_yield(double strain, double strain_rate, double temp) const {
    double T_h = (temp - T_t) / (T_m - T_t);
    double f = 1.0;
    if (strain_rate > eps_0) f = (1.0 + C * std::log(strain_rate / eps_0));
    return (A + B * std::pow(strain, n)) * f * (1.0 - std::pow(T_h, jm));
  }
  // Material.cpp:59-64 Hollomon::CalcYieldStress
  double hol_yield(double strain) const {
    if (strain + eps0 > eps1) return K * std::pow(strain + eps0, m);
    return sy0;
  }
};

struct Amplitude {  // Domain.h:69-89
  int id;
  std::vector<double> time, value;
  double at(double t) const {
    int i = (int)time.size() - 1;
    bool end = false;
    while (!end) { i--; if (i == 0 || t > time[i]) end = true; }
    return value[i] + (value[i + 1] - value[i]) / (time[i + 1] - time[i]) * (t - time[i]);
  }
};

struct BC { int zone; V3 value, value_ang; int value_type; int amp_id; double amp_factor; };

struct Element { int node[3]; V3 centroid, normal; double pplane = 0, radius = 0; int nfar = 0; };
struct TriMesh {  // Mesh.h:44-75
  std::vector<V3> node, node_v;
  std::vector<Element> element;
  int id = 0, dimension = 3;
  V3 m_v = v3(0, 0, 0), m_w = v3(0, 0, 0);
  // Mesh.cpp:229-240 CalcNormals (3D)
  void calc_normals() {
    for (auto& e : element) {
      V3 u = sub(node[e.node[1]], node[e.node[0]]);
      V3 w = sub(node[e.node[2]], node[e.node[0]]);
      V3 c = cross(u, w);
      double nn = norm(c);
      e.normal = v3(c.c[0] / nn, c.c[1] / nn, c.c[2] / nn);
    }
  }
  // Mesh.cpp:70-78 CalcCentroids
  void calc_centroids() {
    for (auto& e : element) {
      V3 c = v3(0, 0, 0);
      for (int i = 0; i < dimension; ++i) c = add(c, node[e.node[i]]);
      e.centroid = v3(c.c[0] / dimension, c.c[1] / dimension, c.c[2] / dimension);
    }
  }
  // Mesh.cpp:222-227 UpdatePlaneCoeff
  void update_plane_coeff() { for (auto& e : element) e.pplane = dot(node[e.node[e.nfar]], e.normal); }
  // Mesh.cpp:273-293 Update
  void update(double dt) {
    for (size_t n = 0; n < node.size(); ++n) {
      V3 vr = cross(m_w, node[n]);
      node_v[n] = add(m_v, vr);
      node[n] = add(node[n], scl(dt, node_v[n]));
    }
    calc_centroids();
    calc_normals();
    update_plane_coeff();
  }
};

// ----------------------------------------------------------------------------
struct Domain {
  int dim = 3;
  // Domain.cpp:78-175 defaults
  double Cellfac = 2.0;
  int ts_nb_inc = 5;
  int pl_heating = 0, thermal_solver = 0, contact = 0, contact_mesh_auto_update = 1;
  double pl_work_heat_frac = 0.9;
  double friction_sta = 0.0, friction_dyn = 0.0, PFAC = 0.0, DFAC = 0.0;
  int64_t dyn_friction_count = 0;  // contact-pair evaluations that took the dynamic-friction branch
  int nan_count = 0;               // particles with a non-finite position at the last search
  int contact_alg = 0;
  double DomMax[3] = {-100000000000.0, -100000000000.0, -100000000000.0};
  double DomMin[3] = {100000000000.0, 100000000000.0, 100000000000.0};
  int mode = 0;       // 0 canonical, 1 reference-structured
  int integrator = 0; // 0 kick-drift (SolverKickDrift.cpp), 1 leapfrog (SolverLeapfrog.cpp)
  // adaptive time step (Domain.cpp:107-170 defaults; Domain.h:326-456)
  int auto_ts = 0, auto_ts_acc = 0, auto_ts_cont = 0;
  double CFL = 0.7, sqrt_h_a = 0.0025, deltatint = 0, deltatmin = 0;
  int h_update = 0;   // Domain::h_update (Domain.cpp:149; JSON "smoothlenUpdate", WeldForm.cpp:377-389)
  int grad_corr = 0;  // Domain::gradKernelCorr (Domain.cpp:130; forces the locking sums, SolverKickDrift.cpp:107-110)
  int nthreads = 1;

  // particles (SoA, original order)
  int N = 0, solid_part_count = -1;
  std::vector<V3> x, v, a, x_prev, disp, normal, contforce;
  std::vector<double> rho, rho0, mass, h, hini, Cs, P0, G, pressure, pl_strain, delta_pl_strain, sigmay, Ep,
      eff_strain_rate, T, dTdt, k_T, cp_T, th_exp, q_plheat, q_conv, q_source, q_cont_conv, ps_energy, alpha,
      T_inf, h_conv,
      beta, TI, TIn, TIInitDist, dDensity, cont_stiff, delta_cont, dkin, dint;
  std::vector<M3> sigma, tau, srate, rrate, strain, strain_pl, strain_pl_incr, TIR, gcm;
  std::vector<int> ID, ID_orig, not_write_surf, is_free, material_idx, mat, model, fail_crit, pres_eq, Nb, mesh_of, elem_of,
      thermal_bc;

  std::vector<Material> materials;
  std::vector<Amplitude> amps;
  std::vector<BC> bcs;
  std::vector<TriMesh> meshes;
  std::vector<int> first_fem, contact_surf_id;
  std::vector<V3> m_contact_force;
  int id_free_surf = -999999;

  // cells (Neighbour.cpp:10-139)
  double BLPF[3] = {0, 0, 0}, TRPR[3] = {0, 0, 0}, CellSize[3] = {0, 0, 0}, hmax = 0;
  int CellNo[3] = {0, 0, 0};
  bool cells_ready = false;

  // neighbour data
  std::vector<std::pair<int, int>> sm_pairs;          // canonical mode: (min,max) sorted
  std::vector<std::vector<std::pair<int, int>>> tp;    // reference mode: per-thread SMPairs
  std::vector<std::vector<std::pair<int, int>>> trig;  // per-thread RIGPairs
  std::vector<std::pair<int, int>> rig_pairs, cont_pairs;
  std::vector<int64_t> nb_off;                         // canonical CSR
  std::vector<int> nb_idx;
  std::vector<int64_t> cp_off;                         // contact CSR (solid -> mesh)
  std::vector<int> cp_idx;
  // reference-mode Nishimura tables (Neighbour.cpp:570-694)
  std::vector<int> ipair, jpair;
  std::vector<int> Anei, Aref;
  std::vector<V3> pair_force;
  std::vector<double> pair_dens;
  std::vector<M3> pair_sr, pair_rr;

  // solver state (SolverKickDrift.cpp:23-115)
  bool prepared = false;
  double Time = 0, deltat = 0, prev_deltat = 0;
  bool isfirst = true, isyielding = false, nb_cleared = false, check_nb_every_time = false;
  int ts_i = 0;
  // Batched specimens: particle -> specimen, and each specimen's own rebuild
  // schedule (the SolverKickDrift.cpp:153-186, 315-324 state of a run of that
  // specimen alone).  A specimen that does not search keeps its rows.
  struct SpecSched { bool isyielding = false, nb_cleared = true; int ts_i = 0; double max_pl = 0; int64_t searches = 0; };
  int nspec = 0;
  std::vector<int> spec_of;
  std::vector<int64_t> spec_first, spec_count;
  std::vector<SpecSched> spec;
  int64_t steps = 0, nb_searches = 0;
  double int_energy_sum = 0, kin_energy_sum = 0, plastic_work = 0, contact_force_sum = 0, contact_reaction_sum = 0,
         ext_forces_work = 0, m_maxT = 0, m_minT = 0, max_pl = 0;
  int surface_count = 0;
  double tangent_mismatch = 0;  // largest relative value difference seen by the tangent run

  void push_particle(int tag, const V3& xx, double m0, double dens, double hh, bool fixed) {
    // Particle.cpp:28-157 constructor defaults
    x.push_back(xx); v.push_back(v3(0, 0, 0)); a.push_back(v3(0, 0, 0)); x_prev.push_back(xx);
    disp.push_back(v3(0, 0, 0)); normal.push_back(v3(0, 0, 0)); contforce.push_back(v3(0, 0, 0));
    rho.push_back(dens); rho0.push_back(dens); mass.push_back(m0); h.push_back(hh); hini.push_back(hh); Cs.push_back(0); P0.push_back(0);
    G.push_back(0); pressure.push_back(0); pl_strain.push_back(0); delta_pl_strain.push_back(0); sigmay.push_back(0);
    Ep.push_back(0); eff_strain_rate.push_back(0); T.push_back(0); dTdt.push_back(0); k_T.push_back(0);
    cp_T.push_back(0); th_exp.push_back(0); q_plheat.push_back(0); q_conv.push_back(0); q_source.push_back(0);
    T_inf.push_back(0); h_conv.push_back(0); thermal_bc.push_back(0);  // Thermal_BC = TH_BC_NONE (Particle.cpp:102)
    q_cont_conv.push_back(0); ps_energy.push_back(0); alpha.push_back(0); beta.push_back(0); TI.push_back(0);
    TIn.push_back(4.0); TIInitDist.push_back(0); dDensity.push_back(0); cont_stiff.push_back(0); delta_cont.push_back(0);
    dkin.push_back(0); dint.push_back(0);
    sigma.push_back(zero3()); tau.push_back(zero3()); srate.push_back(zero3()); rrate.push_back(zero3());
    strain.push_back(zero3()); strain_pl.push_back(zero3()); strain_pl_incr.push_back(zero3()); TIR.push_back(zero3());
    { M3 I = zero3(); at(I, 0, 0) = at(I, 1, 1) = at(I, 2, 2) = 1.0; gcm.push_back(I); }
    ID.push_back(tag); ID_orig.push_back(tag); not_write_surf.push_back(0); is_free.push_back(fixed ? 0 : 1);
    material_idx.push_back(0); mat.push_back(-1); model.push_back(0); fail_crit.push_back(0); pres_eq.push_back(0);
    Nb.push_back(0); mesh_of.push_back(-1); elem_of.push_back(-1);
    ++N;
  }
  bool is_mesh(int p) const { return mesh_of[p] >= 0; }

  // -------------------------------------------------------------- generators
  // Domain.cpp:674-689 calcHalfPartCount
  static int half_count(double r, double R, int xinc) {
    int ypartcount = -1;
    if (xinc > 0) {
      ypartcount = 1;
      double yp = r;
      double xp = r + (double)(xinc - 1) * 2. * r;
      double rad = std::sqrt(yp * yp + xp * xp);
      while (rad <= R - r) { yp += 2. * r; rad = std::sqrt(yp * yp + xp * xp); ypartcount++; }
      ypartcount -= 1;
    }
    return ypartcount;
  }
  // Domain.cpp:708-860 AddCylinderLength (3D, no ghost rows)
  int add_cylinder(int tag, V3 V, double Rxy, double Lz, double r, double dens, double hh, bool fixed) {
    int numpartxy = half_count(r, Rxy, 1);
    double zp = V.c[2] + r;
    while (zp <= (V.c[2] + Lz - r)) {
      double yp = V.c[1] - r - (2. * r * (numpartxy - 1));
      int numypart = 2 * numpartxy, yinc = numpartxy, yinc_sign = -1;
      for (int j = 0; j < numypart; j++) {
        int numxpart = half_count(r, Rxy, yinc);
        double xp = V.c[0] - r - (2. * r * (numxpart - 1));
        for (int i = 0; i < 2 * numxpart; i++) { push_particle(tag, v3(xp, yp, zp), 0.0, dens, hh, fixed); xp += 2. * r; }
        yp += 2. * r;
        yinc += yinc_sign;
        if (yinc < 1) { yinc = 1; yinc_sign = 1; }
      }
      zp += 2. * r;
    }
    solid_part_count = N;
    double Vol = PI * Rxy * Rxy * Lz;
    double Mass = Vol * dens / N;
    for (int i = 0; i < N; ++i) mass[i] = Mass;
    return WF_OK;
  }
  // Domain.cpp:326-599 AddBoxLength (3D branches)
  int add_box(int tag, V3 V, double Lx, double Ly, double Lz, double r, double dens, double hh, int type, int rotation,
              bool random, bool fixed) {
    if (!(type == 0 || type == 1)) return set_err(WF_ERR_ARG, "AddBoxLength: packing type must be 0 or 1");
    if (!(rotation == 0 || rotation == 90)) return set_err(WF_ERR_ARG, "AddBoxLength: rotation must be 0 or 90");
    int PrePS = N;
    double qin = 0.03;
    srand(100);
    double xq, yq, xp, yp;
    if (type == 0) {
      double zq, zp;
      size_t k = 0;
      zp = V.c[2];
      while (zp <= (V.c[2] + Lz - r)) {
        size_t j = 0;
        yp = V.c[1];
        while (yp <= (V.c[1] + Ly - r)) {
          size_t i = 0;
          xp = V.c[0];
          while (xp <= (V.c[0] + Lx - r)) {
            if ((k % 2 != 0) && (j % 2 != 0)) xq = V.c[0] + (2 * i + (j % 2) + (k % 2) - 1) * r;
            else xq = V.c[0] + (2 * i + (j % 2) + (k % 2) + 1) * r;
            yq = V.c[1] + (std::sqrt(3.0) * (j + (1.0 / 3.0) * (k % 2)) + 1) * r;
            zq = V.c[2] + ((2 * std::sqrt(6.0) / 3) * k + 1) * r;
            if (random) {
              double rx = qin * r * double(rand()) / RAND_MAX; double ry = qin * r * double(rand()) / RAND_MAX;
              double rz = qin * r * double(rand()) / RAND_MAX;
              push_particle(tag, v3(xq + rx, yq + ry, zq + rz), 0.0, dens, hh, fixed);
            } else push_particle(tag, v3(xq, yq, zq), 0.0, dens, hh, fixed);
            i++;
            if ((k % 2 != 0) && (j % 2 != 0)) xp = V.c[0] + (2 * i + (j % 2) + (k % 2) - 1) * r;
            else xp = V.c[0] + (2 * i + (j % 2) + (k % 2) + 1) * r;
          }
          j++;
          yp = V.c[1] + (std::sqrt(3.0) * (j + (1.0 / 3.0) * (k % 2)) + 1) * r;
        }
        k++;
        zp = V.c[2] + ((2 * std::sqrt(6.0) / 3) * k + 1) * r;
      }
    } else {
      double zq, zp;
      size_t k = 0;
      zp = V.c[2];
      while (zp <= (V.c[2] + Lz - r)) {
        size_t j = 0;
        yp = V.c[1];
        while (yp <= (V.c[1] + Ly - r)) {
          size_t i = 0;
          xp = V.c[0];
          while (xp <= (V.c[0] + Lx - r)) {
            xq = V.c[0] + (2.0 * i + 1) * r;
            yq = V.c[1] + (2.0 * j + 1) * r;
            zq = V.c[2] + (2.0 * k + 1) * r;
            if (random) {
              double rx = qin * r * double(rand()) / RAND_MAX; double ry = qin * r * double(rand()) / RAND_MAX;
              double rz = qin * r * double(rand()) / RAND_MAX;
              push_particle(tag, v3(xq + rx, yq + ry, zq + rz), 0.0, dens, hh, fixed);
            } else push_particle(tag, v3(xq, yq, zq), 0.0, dens, hh, fixed);
            i++;
            xp = V.c[0] + (2 * i + 1) * r;
          }
          j++;
          yp = V.c[1] + (2.0 * j + 1) * r;
        }
        k++;
        zp = V.c[2] + (2.0 * k + 1) * r;
      }
    }
    V3 Max = V;
    for (int i = PrePS; i < N; i++)
      for (int d = 0; d < 3; ++d) if (x[i].c[d] > Max.c[d]) Max.c[d] = x[i].c[d];
    for (int d = 0; d < 3; ++d) Max.c[d] += r;
    V3 tmp = sub(Max, V);
    double Mass = tmp.c[0] * tmp.c[1] * tmp.c[2] * dens / (N - PrePS);
    for (int i = 0; i < N; ++i) mass[i] = Mass;  // the reference assigns every particle (Domain.cpp:461-469)
    solid_part_count = N;
    return WF_OK;
  }
  // Domain.cpp:691-706 AssignZone
  int64_t assign_zone(const V3& s, const V3& e, int id) {
    int64_t cnt = 0;
    for (int p = 0; p < N; ++p) {
      bool inc = true;
      for (int d = 0; d < 3; ++d) if (x[p].c[d] < s.c[d] || x[p].c[d] > e.c[d]) inc = false;
      if (inc) { ID[p] = id; not_write_surf[p] = 1; cnt++; }
    }
    return cnt;
  }
  // Mesh.cpp:82-203 AxisPlaneMesh (3D), Mesh.cpp:206-220 CalcSpheres,
  // Contact.cpp:10-38 AddTrimeshParticles
  int add_plane(int axis, bool posit, V3 p1, V3 p2, int dens, double hfac, int zone) {
    TriMesh M;
    V3 p = sub(p2, p1);
    int dir[3];
    if (axis == 0) { dir[0] = 1; dir[1] = 2; } else if (axis == 1) { dir[0] = 0; dir[1] = 2; } else { dir[0] = 0; dir[1] = 1; }
    dir[2] = axis;
    double x3 = p1.c[dir[2]], x2 = p1.c[dir[1]];
    double dl = p.c[dir[0]] / dens;
    for (int j = 0; j < dens + 1; j++) {
      double x1 = p1.c[dir[0]];
      for (int i = 0; i < dens + 1; i++) {
        V3 q; q.c[dir[0]] = x1; q.c[dir[1]] = x2; q.c[dir[2]] = x3;
        M.node.push_back(q); M.node_v.push_back(v3(0, 0, 0));
        x1 += dl;
      }
      x2 += dl;
    }
    for (int j = 0; j < dens; j++)
      for (int i = 0; i < dens; i++) {
        int n0 = (dens + 1) * j + i, n1 = n0 + 1, n2 = (dens + 1) * (j + 1) + i, n3 = n2 + 1;
        int ec[2][3];
        if (posit) { ec[0][0] = n0; ec[0][1] = n1; ec[0][2] = n2; ec[1][0] = n1; ec[1][1] = n3; ec[1][2] = n2; }
        else { ec[0][0] = n0; ec[0][1] = n2; ec[0][2] = n1; ec[1][0] = n1; ec[1][1] = n2; ec[1][2] = n3; }
        for (int e = 0; e < 2; ++e) {
          Element el;
          for (int k = 0; k < 3; ++k) el.node[k] = ec[e][k];
          V3 s = add(add(M.node[ec[e][0]], M.node[ec[e][1]]), M.node[ec[e][2]]);
          el.centroid = v3(s.c[0] / 3., s.c[1] / 3., s.c[2] / 3.);
          M.element.push_back(el);
        }
      }
    M.calc_normals();
    if (posit) for (auto& e : M.element) e.normal = scl(-1.0, e.normal);
    for (auto& e : M.element) {  // CalcSpheres
      double mx = 0.;
      for (int n = 0; n < M.dimension; n++) {
        V3 rv = sub(M.node[e.node[n]], e.centroid);
        if (norm(rv) > mx) mx = norm(rv);
        e.nfar = n;
      }
      e.radius = mx;
    }
    M.update_plane_coeff();
    M.id = zone;
    int mi = (int)meshes.size();
    first_fem.push_back(N);
    contact_surf_id.push_back(zone);
    for (size_t e = 0; e < M.element.size(); ++e) {
      double hh = (double)(float)hfac * M.element[e].radius;  // hfac is a float parameter (Contact.cpp:10)
      push_particle(zone, M.element[e].centroid, 0.0, 0.0, hh, false);
      normal[N - 1] = M.element[e].normal;
      elem_of[N - 1] = (int)e;
      mesh_of[N - 1] = mi;
    }
    meshes.push_back(M);
    m_contact_force.push_back(v3(0, 0, 0));
    return mi;
  }

  // -------------------------------------------------------------- cells
  // Neighbour.cpp:10-139 CellInitiate (3D, non-periodic)
  int cell_initiate() {
    if (!(std::sqrt(TRPR[0] * TRPR[0] + TRPR[1] * TRPR[1] + TRPR[2] * TRPR[2]) > 0.0) &&
        !(std::sqrt(BLPF[0] * BLPF[0] + BLPF[1] * BLPF[1] + BLPF[2] * BLPF[2]) > 0.0)) {
      for (int d = 0; d < 3; ++d) { BLPF[d] = x[0].c[d]; TRPR[d] = x[0].c[d]; }
      hmax = h[0];
      for (int i = 0; i < N; i++) {
        for (int d = 0; d < 3; ++d) {
          if (x[i].c[d] > TRPR[d]) TRPR[d] = x[i].c[d];
          if (x[i].c[d] < BLPF[d]) BLPF[d] = x[i].c[d];
        }
        if (h[i] > hmax) hmax = h[i];
      }
    }
    for (int d = 0; d < 3; ++d) { if (DomMax[d] > TRPR[d]) TRPR[d] = DomMax[d]; if (DomMin[d] < BLPF[d]) BLPF[d] = DomMin[d]; }
    for (int d = 0; d < 3; ++d) { TRPR[d] += hmax / 2; BLPF[d] -= hmax / 2; }
    for (int d = 0; d < 3; ++d) {
      double t = (TRPR[d] - BLPF[d]) / (Cellfac * hmax);
      if (double(std::ceil(t) - t) < (hmax / 10.0)) CellNo[d] = int(std::ceil(t));
      else CellNo[d] = int(std::floor(t));
      if (CellNo[d] <= 0) return set_err(WF_ERR_ARG, "CellInitiate: domain extent smaller than one cell");
    }
    for (int d = 0; d < 3; ++d) CellSize[d] = (TRPR[d] - BLPF[d]) / CellNo[d];
    cells_ready = true;
    return WF_OK;
  }
  // Neighbour.cpp:183-227 ListGenerate cell index (3D, clamped)
  void cell_of(int a, int c[3]) const {
    for (int d = 0; d < 3; ++d) {
      int q = (int)(std::floor((x[a].c[d] - BLPF[d]) / CellSize[d]));
      if (q < 0) q = 0;
      if (q >= CellNo[d]) q = CellNo[d] - 1;
      c[d] = q;
    }
  }
  // Neighbour.cpp:361-372 CheckRadius
  bool check_radius(int p1, int p2) const {
    double hh = (h[p1] + h[p2]) / 2;
    V3 xij = sub(x[p1], x[p2]);
    double rij = norm(xij);
    return (rij / hh) <= Cellfac;
  }
  bool is_contact_id(int id) const {
    for (int s : contact_surf_id) if (id == s) return true;
    return false;
  }
  // Neighbour.cpp:374-417 AllocateNbPair; returns 1 = SM pair, 2 = RIG pair, 0 = none
  int classify_pair(int t1, int t2) const {
    if (contact) {
      bool isc = false;
      for (size_t m = 0; m < contact_surf_id.size(); m++)
        if (ID[t1] == contact_surf_id[m] || ID[t2] == contact_surf_id[m]) isc = true;
      if (isc) {
        if (ID[t1] == id_free_surf || ID[t2] == id_free_surf) return 2;
        return 0;
      }
    }
    if (check_radius(t1, t2)) {
      if (is_free[t1] || is_free[t2]) {
        if (material_idx[t1] == material_idx[t2]) {
          if (is_free[t1] && is_free[t2]) return 1;
        }
      }
    }
    return 0;
  }
  // Neighbour.cpp:141-257 ListGenerate + 346-477 MainNeighbourSearch with
  // YZPlaneCellsNeighbourSearch (half stencil over head-of-chain lists).
  void search_linked_list() {
    int nx = CellNo[0], ny = CellNo[1], nz = CellNo[2];
    std::vector<int> HOC((size_t)nx * ny * nz, -1), LL(N, -1);
    auto cidx = [&](int i, int j, int k) { return ((size_t)i * ny + j) * nz + k; };
    for (int a = 0; a < N; a++) {
      int c[3]; cell_of(a, c);
      size_t ci = cidx(c[0], c[1], c[2]);
      LL[a] = HOC[ci];
      HOC[ci] = a;
    }
    int nt = (mode == 1) ? nthreads : 1;
    tp.assign(nt, {});
    trig.assign(nt, {});
    auto slab = [&](int q1, int T) {
      auto alloc = [&](int t1, int t2) {
        int c = classify_pair(t1, t2);
        if (c == 1) tp[T].push_back({t1, t2});
        else if (c == 2) trig[T].push_back({t1, t2});
      };
      for (int q3 = 0; q3 < nz; q3++)
        for (int q2 = 0; q2 < ny; q2++) {
          int t1 = HOC[cidx(q1, q2, q3)];
          while (t1 != -1) {
            int t2 = LL[t1];
            while (t2 != -1) { alloc(t1, t2); t2 = LL[t2]; }
            if (q1 + 1 < nx) { t2 = HOC[cidx(q1 + 1, q2, q3)]; while (t2 != -1) { alloc(t1, t2); t2 = LL[t2]; } }
            if (q2 + 1 < ny)
              for (int i = q1 - 1; i <= q1 + 1; i++)
                if (i < nx && i >= 0) { t2 = HOC[cidx(i, q2 + 1, q3)]; while (t2 != -1) { alloc(t1, t2); t2 = LL[t2]; } }
            if (q3 + 1 < nz)
              for (int j = q2 - 1; j <= q2 + 1; j++)
                for (int i = q1 - 1; i <= q1 + 1; i++)
                  if (i < nx && i >= 0 && j < ny && j >= 0) {
                    t2 = HOC[cidx(i, j, q3 + 1)];
                    while (t2 != -1) { alloc(t1, t2); t2 = LL[t2]; }
                  }
            t1 = LL[t1];
          }
        }
    };
    if (nt > 1) {
#pragma omp parallel for schedule(dynamic) num_threads(nt)
      for (int q1 = 0; q1 < nx; q1++) {
        int T = 0;
#ifdef _OPENMP
        T = omp_get_thread_num();
#endif
        slab(q1, T);
      }
    } else {
      for (int q1 = 0; q1 < nx; q1++) slab(q1, 0);
    }
  }
  // Canonical CSR from the pair set: row i holds j > i ascending, then j < i
  // ascending (the Anei layout of Neighbour.cpp:672-675 with a fixed order).
  int build_canonical() {
    std::vector<int64_t> cnt(N + 1, 0);
    sm_pairs.clear();
    for (auto& t : tp) for (auto& pr : t) sm_pairs.push_back({std::min(pr.first, pr.second), std::max(pr.first, pr.second)});
    for (auto& pr : sm_pairs) { cnt[pr.first + 1]++; cnt[pr.second + 1]++; }
    nb_off.assign(N + 1, 0);
    for (int i = 0; i < N; ++i) nb_off[i + 1] = nb_off[i] + cnt[i + 1];
    nb_idx.assign(nb_off[N], 0);
    std::vector<int64_t> cur(nb_off.begin(), nb_off.end() - 1);
    for (auto& pr : sm_pairs) { nb_idx[cur[pr.first]++] = pr.second; nb_idx[cur[pr.second]++] = pr.first; }
    int over = 0;
    for (int i = 0; i < N; ++i) {
      auto b = nb_idx.begin() + nb_off[i], e = nb_idx.begin() + nb_off[i + 1];
      std::sort(b, e, [i](int p, int q) { return (uint32_t)(p - i - 1) < (uint32_t)(q - i - 1); });
      Nb[i] = (int)(nb_off[i + 1] - nb_off[i]);  // SaveNeighbourData, Neighbour.cpp:499-532
      if (Nb[i] > MAX_NB_PER_PART) over = 1;
    }
    rig_pairs.clear();
    for (auto& t : trig) for (auto& pr : t) rig_pairs.push_back(pr);
    if (over) return set_err(WF_ERR_NBR_OVERFLOW, "a particle has more than 100 neighbours (MAX_NB_PER_PART)");
    return WF_OK;
  }
  // Neighbour.cpp:617-694 CalcPairPosList for the reference-structured mode.
  void build_nishimura() {
    int64_t pc = 0;
    std::vector<int64_t> first(tp.size(), 0);
    for (size_t k = 0; k < tp.size(); ++k) { first[k] = pc; pc += (int64_t)tp[k].size(); }
    pair_force.resize(pc); pair_dens.resize(pc); pair_sr.resize(pc); pair_rr.resize(pc);
    ipair.assign(N, 0); jpair.assign(N, 0);
    Anei.assign((size_t)N * MAX_NB_PER_PART, 0); Aref.assign((size_t)N * MAX_NB_PER_PART, 0);
    for (size_t k = 0; k < tp.size(); ++k)
      for (size_t pp = 0; pp < tp[k].size(); ++pp) {
        int i = std::min(tp[k][pp].first, tp[k][pp].second), j = std::max(tp[k][pp].first, tp[k][pp].second);
        if (ipair[i] < MAX_NB_PER_PART && jpair[j] < MAX_NB_PER_PART) {
          Anei[(size_t)i * MAX_NB_PER_PART + ipair[i]] = j;
          Anei[(size_t)j * MAX_NB_PER_PART + MAX_NB_PER_PART - 1 - jpair[j]] = i;
          Aref[(size_t)i * MAX_NB_PER_PART + ipair[i]] = (int)(first[k] + pp);
          Aref[(size_t)j * MAX_NB_PER_PART + MAX_NB_PER_PART - 1 - jpair[j]] = (int)(first[k] + pp);
        }
        ipair[i]++; jpair[j]++;
      }
  }
  // Domain::CalcGradCorrMatrix (Domain.cpp:1832-1940): per particle
  // M_i = -sum_j (m_j/rho_j) (GK x_ij) (x) x_ij over its neighbours (canonical
  // row order), then gradCorrM_i = InvLog(M_i), the identity where the
  // determinant is below 1e-10 (matvec.h:673-693).
  void calc_grad_corr() {
    int mx = contact ? first_fem[0] : N;
    for (int i = 0; i < mx; i++) {
      M3 t = zero3();
      for (int64_t k = nb_off[i]; k < nb_off[i + 1]; ++k) {
        int j = nb_idx[k];
        int P1 = std::min(i, j), P2 = std::max(i, j);
        V3 xij = sub(x[P1], x[P2]);
        double hh = (h[P1] + h[P2]) / 2.0;
        double GK = grad_kernel(dim, norm(xij) / hh, hh);
        V3 g = scl(GK, xij);
        double f = mass[j] / rho[j];
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b) at(t, a, b) = at(t, a, b) - f * (g.c[a] * xij.c[b]);
      }
      double det = at(t, 0, 0) * (at(t, 1, 1) * at(t, 2, 2) - at(t, 1, 2) * at(t, 2, 1)) -
                   at(t, 0, 1) * (at(t, 1, 0) * at(t, 2, 2) - at(t, 1, 2) * at(t, 2, 0)) +
                   at(t, 0, 2) * (at(t, 1, 0) * at(t, 2, 1) - at(t, 1, 1) * at(t, 2, 0));
      M3 m;
      if (std::fabs(det) < 1.0e-10) {
        m = zero3(); at(m, 0, 0) = at(m, 1, 1) = at(m, 2, 2) = 1.0;
      } else {
        at(m, 0, 0) = (at(t, 1, 1) * at(t, 2, 2) - at(t, 1, 2) * at(t, 2, 1)) / det;
        at(m, 0, 1) = (at(t, 0, 2) * at(t, 2, 1) - at(t, 0, 1) * at(t, 2, 2)) / det;
        at(m, 0, 2) = (at(t, 0, 1) * at(t, 1, 2) - at(t, 0, 2) * at(t, 1, 1)) / det;
        at(m, 1, 0) = (at(t, 1, 2) * at(t, 2, 0) - at(t, 1, 0) * at(t, 2, 2)) / det;
        at(m, 1, 1) = (at(t, 0, 0) * at(t, 2, 2) - at(t, 0, 2) * at(t, 2, 0)) / det;
        at(m, 1, 2) = (at(t, 0, 2) * at(t, 1, 0) - at(t, 0, 0) * at(t, 1, 2)) / det;
        at(m, 2, 0) = (at(t, 1, 0) * at(t, 2, 1) - at(t, 1, 1) * at(t, 2, 0)) / det;
        at(m, 2, 1) = (at(t, 0, 1) * at(t, 2, 0) - at(t, 0, 0) * at(t, 2, 1)) / det;
        at(m, 2, 2) = (at(t, 0, 0) * at(t, 1, 1) - at(t, 0, 1) * at(t, 1, 0)) / det;
      }
      gcm[i] = m;
    }
  }
  // Corrected kernel gradient of end e of the pair (P1, P2):
  // Mult(GK * gradCorrM_e, x12) (InteractionAlt.cpp:114-132).
  V3 corr_grad(int e, double GK, const V3& x12) const {
    M3 G;
    for (int k = 0; k < 9; ++k) G.m[k] = GK * gcm[e].m[k];
    V3 r;
    for (int k = 0; k < 3; ++k) r.c[k] = x12.c[0] * at(G, k, 0) + x12.c[1] * at(G, k, 1) + x12.c[2] * at(G, k, 2);
    return r;
  }

  int neighbour_search() {
    if (!cells_ready) return set_err(WF_ERR_STATE, "neighbour search before the solver prologue");
    // particles with a non-finite coordinate at this search (reported only;
    // the linked-list search bins them into clamped cells as the reference does)
    nan_count = 0;
    for (int i = 0; i < N; ++i)
      if (!(std::isfinite(x[i].c[0]) && std::isfinite(x[i].c[1]) && std::isfinite(x[i].c[2]))) ++nan_count;
    search_linked_list();
    int rc = build_canonical();
    if (mode == 1) build_nishimura();
    nb_searches++;
    nb_cleared = false;
    return rc;
  }

  // Domain.cpp:1415-1491 CalculateSurface (pairs from the current list)
  int calculate_surface(int id) {
    id_free_surf = id;
    double totmass = 0.;
    for (int i = 0; i < N; i++) totmass += mass[i];
    totmass /= N;
    int maxid = contact ? first_fem[0] : N;
    for (int i = 0; i < maxid; i++) { normal[i] = v3(0, 0, 0); ID[i] = ID_orig[i]; }
    // Eqn 3-112 Fraser: n_i = sum_j m_j (x_i - x_j), summed in canonical row order
    for (int i = 0; i < maxid; i++) {
      V3 acc = v3(0, 0, 0);
      for (int64_t k = nb_off[i]; k < nb_off[i + 1]; ++k) {
        int j = nb_idx[k];
        acc = add(acc, scl(mass[j], sub(x[i], x[j])));
      }
      normal[i] = acc;
    }
    int max_nb = 46;
    int surf = 0;
    for (int i = 0; i < maxid; i++) {
      normal[i] = scl(1. / totmass, normal[i]);
      if (norm(normal[i]) >= 0.25 * h[i] && Nb[i] <= max_nb) {
        if (!not_write_surf[i]) ID[i] = id;
        surf++;
      }
    }
    surface_count = surf;
    if (surf == 0) return set_err(WF_ERR_STATE, "No external particles found. Please check particle masses");
    return WF_OK;
  }
  // Contact.cpp:57-132 ContactNbSearch -> canonical contact CSR
  void contact_nb_search() {
    cont_pairs.clear();
    for (auto& pr : rig_pairs) {
      int P1 = pr.first, P2 = pr.second;
      bool isc = is_contact_id(ID[P1]) || is_contact_id(ID[P2]);
      if (isc && (ID[P1] == id_free_surf || ID[P2] == id_free_surf)) {
        if (norm(sub(x[P1], x[P2])) < (h[P1] + h[P2])) cont_pairs.push_back(pr);
      }
    }
    rig_pairs.clear();
    // Orient (solid, mesh) and order by solid then mesh index.
    std::vector<std::pair<int, int>> sp;
    for (auto& pr : cont_pairs) {
      bool first_is_mesh = is_contact_id(ID[pr.first]);
      int s = first_is_mesh ? pr.second : pr.first, m = first_is_mesh ? pr.first : pr.second;
      sp.push_back({s, m});
    }
    std::sort(sp.begin(), sp.end());
    cp_off.assign(N + 1, 0);
    for (auto& q : sp) cp_off[q.first + 1]++;
    for (int i = 0; i < N; ++i) cp_off[i + 1] += cp_off[i];
    cp_idx.resize(sp.size());
    for (size_t k = 0; k < sp.size(); ++k) cp_idx[k] = sp[k].second;
  }
  int contact_nb_update() {  // Domain.cpp:2481-2487 ContactNbUpdate
    int rc = calculate_surface(1);
    if (rc) return rc;
    contact_nb_search();
    return WF_OK;
  }

  // -------------------------------------------------------------- BCs
  // WeldForm.cpp:51-120 UserAcc
  void general_after() {
    for (int i = 0; i < N; ++i)
      for (auto& bc : bcs) {
        if (ID[i] != bc.zone) continue;
        if (bc.value_type == 0) { a[i] = v3(0, 0, 0); v[i] = bc.value; }
        else {
          for (auto& am : amps)
            if (am.id == bc.amp_id) {
              double val = bc.amp_factor * am.at(Time);
              a[i] = v3(0, 0, 0);
              v[i] = scl(val, bc.value);
            }
        }
      }
    if (contact)
      for (auto& bc : bcs)
        for (auto& M : meshes)
          if (M.id == bc.zone) {
            if (bc.value_type == 0) { M.m_v = bc.value; M.m_w = bc.value_ang; }
            else for (auto& am : amps) if (am.id == bc.amp_id) M.m_v = scl(bc.amp_factor * am.at(Time), bc.value);
          }
  }

  // -------------------------------------------------------------- pair terms
  // InteractionAlt.cpp:35-197, pair (P1, P2) as the Nishimura path orders them.
  V3 pair_accel(int P1, int P2, int corr_end = -1) const {
    double hh = (h[P1] + h[P2]) / 2;
    V3 xij = sub(x[P1], x[P2]);
    double rij = norm(xij);
    double Alpha = (alpha[P1] + alpha[P2]) / 2.0, Beta = (beta[P1] + beta[P2]) / 2.0;
    double di = rho[P1], dj = rho[P2];
    V3 vij = sub(v[P1], v[P2]);
    double GK = grad_kernel(dim, rij / hh, hh);
    double PI_s = 0.0;
    bool has_pi = false;
    if (Alpha != 0.0 || Beta != 0.0) {
      double MUij = hh * dot(vij, xij) / (rij * rij + 0.01 * hh * hh);
      double Cij = 0.5 * (Cs[P1] + Cs[P2]);  // SoundSpeed case 0 returns Cs (Functions.cpp:232-238)
      if (dot(vij, xij) < 0) { PI_s = (Alpha * Cij * MUij + Beta * MUij * MUij) / (0.5 * (di + dj)); has_pi = true; }
    }
    // Tensile instability (InteractionAlt.cpp:102-109):
    // TIij = (W(rij/h) / W(dinit/h))^((n1+n2)/2) (TIR1 + TIR2)
    bool has_ti = TI[P1] > 0.0 || TI[P2] > 0.0;
    double fti = 0.0;
    if (has_ti) {
      double K = kernel_w(dim, rij / hh, hh);
      fti = std::pow((K / kernel_w(dim, (TIInitDist[P1] + TIInitDist[P2]) / (2.0 * hh), hh)), (TIn[P1] + TIn[P2]) / 2.0);
    }
    M3 S;
    double ci = 1.0 / (di * di), cj = 1.0 / (dj * dj);
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l) {
        double s = ci * at(sigma[P1], k, l) + cj * at(sigma[P2], k, l);
        if (has_pi) s = s + PI_s * I3(k, l);
        if (has_ti) s = s + fti * (at(TIR[P1], k, l) + at(TIR[P2], k, l));
        at(S, k, l) = s;
      }
    if (corr_end >= 0) return vecmat(corr_grad(corr_end, GK, xij), S);  // temp_c (InteractionAlt.cpp:166-170)
    return vecmat(scl(GK, xij), S);
  }
  // InteractionAlt.cpp:505-565
  double pair_densinc(int P1, int P2) const {
    double hh = (h[P1] + h[P2]) / 2;
    V3 xij = sub(x[P1], x[P2]);
    double rij = norm(xij);
    V3 vij = sub(v[P1], v[P2]);
    double GK = grad_kernel(dim, rij / hh, hh);
    return dot(vij, scl(GK, xij));
  }
  // InteractionAlt.cpp:283-361
  void pair_rates(int P1, int P2, M3& SR, M3& RR) const {
    double hh = (h[P1] + h[P2]) / 2;
    V3 xij = sub(x[P1], x[P2]);
    double rij = norm(xij);
    V3 vab = sub(v[P1], v[P2]);
    double GK = grad_kernel(dim, rij / hh, hh);
    const double* vb = vab.c; const double* xx = xij.c;
    SR = zero3(); RR = zero3();
    at(SR, 0, 0) = 2.0 * vb[0] * xx[0];
    at(SR, 0, 1) = vb[0] * xx[1] + vb[1] * xx[0];
    at(SR, 0, 2) = vb[0] * xx[2] + vb[2] * xx[0];
    at(SR, 1, 0) = at(SR, 0, 1);
    at(SR, 1, 1) = 2.0 * vb[1] * xx[1];
    at(SR, 1, 2) = vb[1] * xx[2] + vb[2] * xx[1];
    at(SR, 2, 0) = at(SR, 0, 2);
    at(SR, 2, 1) = at(SR, 1, 2);
    at(SR, 2, 2) = 2.0 * vb[2] * xx[2];
    double f = -0.5 * GK;
    for (int k = 0; k < 9; ++k) SR.m[k] = f * SR.m[k];
    at(RR, 0, 1) = vb[0] * xx[1] - vb[1] * xx[0];
    at(RR, 0, 2) = vb[0] * xx[2] - vb[2] * xx[0];
    at(RR, 1, 2) = vb[1] * xx[2] - vb[2] * xx[1];
    at(RR, 1, 0) = -at(RR, 0, 1);
    at(RR, 2, 0) = -at(RR, 0, 2);
    at(RR, 2, 1) = -at(RR, 1, 2);
    for (int k = 0; k < 9; ++k) RR.m[k] = f * RR.m[k];
  }
  // Thermal.cpp:72-131 conduction pair term for (P1, P2)
  double pair_conduction(int P1, int P2, int corr_end = -1) const {
    V3 xij = sub(x[P1], x[P2]);
    double hh = (h[P1] + h[P2]) / 2.0;
    double GK = grad_kernel(dim, norm(xij) / hh, hh);
    double mj = mass[P2], dj = rho[P2];
    V3 g = scl(GK, xij);
    if (corr_end >= 0) {  // Mult(gradCorrM_e, GK x12) (Thermal.cpp:90-107)
      const M3& M = gcm[corr_end];
      V3 c;
      for (int k = 0; k < 3; ++k) c.c[k] = g.c[0] * at(M, k, 0) + g.c[1] * at(M, k, 1) + g.c[2] * at(M, k, 2);
      g = c;
    }
    return mj / dj * 4. * (k_T[P1] * k_T[P2]) / (k_T[P1] + k_T[P2]) * (T[P1] - T[P2]) * dot(xij, g) /
           (norm(xij) * norm(xij));
  }
  // Domain.cpp:1775-1790 kinetic-energy pair term for (P1, P2)
  double pair_kin(int P1, int P2) const {
    V3 xij = sub(x[P1], x[P2]), vij = sub(v[P1], v[P2]);
    double mj = mass[P2], di = rho[P1], dj = rho[P2];
    double hh = (h[P1] + h[P2]) / 2.0;
    double GK = grad_kernel(dim, norm(xij) / hh, hh);
    return 0.5 * mj * (pressure[P1] / (di * di) + pressure[P2] / (dj * dj)) * dot(vij, scl(GK, xij));
  }

  // -------------------------------------------------------------- passes
  // Canonical gather: row entries k in [off[i], off[i+1]); j > i first.
  void pass_accel() {  // CalcAccel + AccelReduction (InteractionAlt.cpp:12-260)
    int ns = solid_part_count;
    if (mode == 1) {
#pragma omp parallel for schedule(static) num_threads(nthreads)
      for (int k = 0; k < (int)tp.size(); ++k) {
        int64_t base = 0;
        for (int q = 0; q < k; ++q) base += (int64_t)tp[q].size();
        for (size_t p = 0; p < tp[k].size(); ++p) {
          int P1 = std::min(tp[k][p].first, tp[k][p].second), P2 = std::max(tp[k][p].first, tp[k][p].second);
          pair_force[base + p] = pair_accel(P1, P2);
        }
      }
#pragma omp parallel for schedule(static) num_threads(nthreads)
      for (int i = 0; i < ns; i++) {
        V3 ai = v3(0, 0, 0);
        const int* an = &Anei[(size_t)i * MAX_NB_PER_PART]; const int* ar = &Aref[(size_t)i * MAX_NB_PER_PART];
        for (int n = 0; n < ipair[i]; n++) ai = add(ai, scl(mass[an[n]], pair_force[ar[n]]));
        for (int n = 0; n < jpair[i]; n++) ai = sub(ai, scl(mass[an[MAX_NB_PER_PART - 1 - n]], pair_force[ar[MAX_NB_PER_PART - 1 - n]]));
        a[i] = ai;
      }
      return;
    }
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int i = 0; i < ns; i++) {
      if (is_mesh(i)) continue;
      V3 ai = v3(0, 0, 0);
      int ce = grad_corr ? i : -1;  // the locking sum's corrected gradient of this end
      for (int64_t k = nb_off[i]; k < nb_off[i + 1]; ++k) {
        int j = nb_idx[k];
        if (j > i) ai = add(ai, scl(mass[j], pair_accel(i, j, ce)));
        else ai = sub(ai, scl(mass[j], pair_accel(j, i, ce)));
      }
      a[i] = ai;
    }
  }
  void pass_density() {  // CalcDensInc + DensReduction (InteractionAlt.cpp:483-640)
    int ns = solid_part_count;
    if (mode == 1) {
#pragma omp parallel for schedule(static) num_threads(nthreads)
      for (int k = 0; k < (int)tp.size(); ++k) {
        int64_t base = 0;
        for (int q = 0; q < k; ++q) base += (int64_t)tp[q].size();
        for (size_t p = 0; p < tp[k].size(); ++p) {
          int P1 = std::min(tp[k][p].first, tp[k][p].second), P2 = std::max(tp[k][p].first, tp[k][p].second);
          pair_dens[base + p] = this->pair_densinc(P1, P2);
        }
      }
#pragma omp parallel for schedule(static) num_threads(nthreads)
      for (int i = 0; i < ns; i++) {
        double dd = 0.;
        const int* an = &Anei[(size_t)i * MAX_NB_PER_PART]; const int* ar = &Aref[(size_t)i * MAX_NB_PER_PART];
        for (int n = 0; n < ipair[i]; n++) dd += mass[an[n]] / rho[an[n]] * pair_dens[ar[n]];
        for (int n = 0; n < jpair[i]; n++) {
          int q = MAX_NB_PER_PART - 1 - n;
          dd += mass[an[q]] / rho[an[q]] * pair_dens[ar[q]];
        }
        dDensity[i] = dd * rho[i];
      }
      return;
    }
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int i = 0; i < ns; i++) {
      if (is_mesh(i)) continue;
      double dd = 0.;
      if (grad_corr) {  // locking form: += m_j (rho_i / rho_j) v12 . Mult(GK M_i, x12) (InteractionAlt.cpp:589-605)
        for (int64_t k = nb_off[i]; k < nb_off[i + 1]; ++k) {
          int j = nb_idx[k];
          int P1 = std::min(i, j), P2 = std::max(i, j);
          double hh = (h[P1] + h[P2]) / 2;
          V3 xij = sub(x[P1], x[P2]);
          double GK = grad_kernel(dim, norm(xij) / hh, hh);
          double t1 = dot(sub(v[P1], v[P2]), corr_grad(i, GK, xij));
          dd += mass[j] * (rho[i] / rho[j]) * t1;
        }
        dDensity[i] = dd;
        continue;
      }
      for (int64_t k = nb_off[i]; k < nb_off[i + 1]; ++k) {
        int j = nb_idx[k];
        double pd = (j > i) ? this->pair_densinc(i, j) : this->pair_densinc(j, i);
        dd += mass[j] / rho[j] * pd;
      }
      dDensity[i] = dd * rho[i];
    }
  }
  void pass_rates() {  // CalcRateTensors + RateTensorsReduction (InteractionAlt.cpp:263-479)
    int ns = solid_part_count;
    if (mode == 1) {
#pragma omp parallel for schedule(static) num_threads(nthreads)
      for (int k = 0; k < (int)tp.size(); ++k) {
        int64_t base = 0;
        for (int q = 0; q < k; ++q) base += (int64_t)tp[q].size();
        for (size_t p = 0; p < tp[k].size(); ++p) {
          int P1 = std::min(tp[k][p].first, tp[k][p].second), P2 = std::max(tp[k][p].first, tp[k][p].second);
          pair_rates(P1, P2, pair_sr[base + p], pair_rr[base + p]);
        }
      }
#pragma omp parallel for schedule(static) num_threads(nthreads)
      for (int i = 0; i < ns; i++) {
        M3& SRi = srate[i]; M3& RRi = rrate[i];
        const int* an = &Anei[(size_t)i * MAX_NB_PER_PART]; const int* ar = &Aref[(size_t)i * MAX_NB_PER_PART];
        auto acc = [&](int q) {
          double mjdj = mass[an[q]] / rho[an[q]];
          for (int c = 0; c < 9; ++c) { SRi.m[c] = SRi.m[c] + mjdj * pair_sr[ar[q]].m[c]; RRi.m[c] = RRi.m[c] + mjdj * pair_rr[ar[q]].m[c]; }
        };
        for (int n = 0; n < ipair[i]; n++) acc(n);
        for (int n = 0; n < jpair[i]; n++) acc(MAX_NB_PER_PART - 1 - n);
      }
      return;
    }
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int i = 0; i < ns; i++) {
      if (is_mesh(i)) continue;
      M3& SRi = srate[i]; M3& RRi = rrate[i];
      if (grad_corr) {  // locking form with corrected gradients (InteractionAlt.cpp:330-350, 425-450)
        for (int64_t k = nb_off[i]; k < nb_off[i + 1]; ++k) {
          int j = nb_idx[k];
          int P1 = std::min(i, j), P2 = std::max(i, j);
          double hh = (h[P1] + h[P2]) / 2;
          V3 xij = sub(x[P1], x[P2]);
          double GK = grad_kernel(dim, norm(xij) / hh, hh);
          V3 vab = sub(v[P1], v[P2]);
          V3 gk = corr_grad(i, GK, xij);
          float mj_dj = mass[j] / rho[j];
          for (int a2 = 0; a2 < 3; ++a2)
            for (int b2 = 0; b2 < 3; ++b2) {
              double g = vab.c[a2] * gk.c[b2], gt = vab.c[b2] * gk.c[a2];
              at(SRi, a2, b2) = at(SRi, a2, b2) + mj_dj * (-0.5 * (g + gt));
              at(RRi, a2, b2) = at(RRi, a2, b2) + mj_dj * (-0.5 * (g - gt));
            }
        }
        continue;
      }
      for (int64_t k = nb_off[i]; k < nb_off[i + 1]; ++k) {
        int j = nb_idx[k];
        M3 SR, RR;
        if (j > i) pair_rates(i, j, SR, RR); else pair_rates(j, i, SR, RR);
        double mjdj = mass[j] / rho[j];
        for (int c = 0; c < 9; ++c) { SRi.m[c] = SRi.m[c] + mjdj * SR.m[c]; RRi.m[c] = RRi.m[c] + mjdj * RR.m[c]; }
      }
    }
  }
  // Particle.cpp:960-1067 CalcStressStrain
  void stress_strain(int i, double dt) {
    double r_ = rho[i];
    pressure[i] = eos0(Cs[i], P0[i], r_, rho0[i]);
    M3& SS = tau[i]; const M3& SR = srate[i]; const M3& RR = rrate[i];
    M3 RRT = trans(RR);
    M3 SRT = matmul(SS, RRT), RS = matmul(RR, SS);
    double dep = 0., sig_trial = 0.;
    double tr = at(SR, 0, 0) + at(SR, 1, 1) + at(SR, 2, 2);
    double s3 = 1.0 / 3.0 * tr;
    double twoG = 2.0 * G[i];
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l)
        at(SS, k, l) = dt * (twoG * (at(SR, k, l) - s3 * I3(k, l)) + at(SRT, k, l) + at(RS, k, l)) + at(SS, k, l);
    eff_strain_rate[i] = std::sqrt(0.5 * ((at(SR, 0, 0) - at(SR, 1, 1)) * (at(SR, 0, 0) - at(SR, 1, 1)) +
                                          (at(SR, 1, 1) - at(SR, 2, 2)) * (at(SR, 1, 1) - at(SR, 2, 2)) +
                                          (at(SR, 2, 2) - at(SR, 0, 0)) * (at(SR, 2, 2) - at(SR, 0, 0))) +
                                   3.0 * (at(SR, 0, 1) * at(SR, 0, 1) + at(SR, 1, 2) * at(SR, 1, 2) + at(SR, 2, 0) * at(SR, 2, 0)));
    const Material* M = (mat[i] >= 0) ? &materials[mat[i]] : nullptr;
    if (fail_crit[i] == 1) {
      double J2 = 0.5 * (at(SS, 0, 0) * at(SS, 0, 0) + 2.0 * at(SS, 0, 1) * at(SS, 1, 0) + 2.0 * at(SS, 0, 2) * at(SS, 2, 0) +
                         at(SS, 1, 1) * at(SS, 1, 1) + 2.0 * at(SS, 1, 2) * at(SS, 2, 1) + at(SS, 2, 2) * at(SS, 2, 2));
      sig_trial = std::sqrt(3.0 * J2);
      double ratio = sigmay[i] / sig_trial;
      double sc = (1.0 < ratio) ? 1.0 : ratio;  // std::min(ratio, 1.0)
      for (int k = 0; k < 9; ++k) SS.m[k] = sc * SS.m[k];
      if (model[i] == 1 && M) sigmay[i] = M->hol_yield(pl_strain[i]);
      else if (model[i] == 2 && M) sigmay[i] = M->jc_yield(pl_strain[i], eff_strain_rate[i], T[i]);
      if (sig_trial > sigmay[i]) {
        if (Ep[i] < 0) Ep[i] = 1. * (M ? M->E : 0.0);
        dep = (sig_trial - sigmay[i]) / (3. * G[i] + Ep[i]);
        pl_strain[i] += dep;
        delta_pl_strain[i] = dep;
        if (model[i] == 0) sigmay[i] += dep * Ep[i];
      }
    }
    M3& Sg = sigma[i];
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l) at(Sg, k, l) = -pressure[i] * I3(k, l) + at(SS, k, l);
    if (dep > 0.0) {
      double f = dep / sigmay[i];
      M3& In = strain_pl_incr[i];
      at(In, 0, 0) = f * (at(Sg, 0, 0) - 0.5 * (at(Sg, 1, 1) + at(Sg, 2, 2)));
      at(In, 1, 1) = f * (at(Sg, 1, 1) - 0.5 * (at(Sg, 0, 0) + at(Sg, 2, 2)));
      at(In, 2, 2) = f * (at(Sg, 2, 2) - 0.5 * (at(Sg, 0, 0) + at(Sg, 1, 1)));
      at(In, 0, 1) = at(In, 1, 0) = 1.5 * f * (at(Sg, 0, 1));
      at(In, 0, 2) = at(In, 2, 0) = 1.5 * f * (at(Sg, 0, 2));
      at(In, 1, 2) = at(In, 2, 1) = 1.5 * f * (at(Sg, 1, 2));
      for (int k = 0; k < 9; ++k) strain_pl[i].m[k] = strain_pl[i].m[k] + In.m[k];
    }
    for (int k = 0; k < 9; ++k) strain[i].m[k] = dt * SR.m[k] + strain[i].m[k];
  }
  // ThermalStuct.cpp:14-39 + Particle.cpp:922-939
  void plastic_work_heat(double dt) {
    if (!pl_heating) return;
    int ns = solid_part_count;
    for (int p = 0; p < ns; p++) {
      if (delta_pl_strain[p] > 0.0) {
        const M3& In = strain_pl_incr[p]; const M3& S = sigma[p];
        double f = 1. / dt;
        M3 d; for (int k = 0; k < 9; ++k) d.m[k] = f * In.m[k];
        q_plheat[p] = at(S, 0, 0) * at(d, 0, 0) + 2.0 * at(S, 0, 1) * at(d, 1, 0) + 2.0 * at(S, 0, 2) * at(d, 2, 0) +
                      at(S, 1, 1) * at(d, 1, 1) + 2.0 * at(S, 1, 2) * at(d, 2, 1) + at(S, 2, 2) * at(d, 2, 2);
      }
      ps_energy[p] += q_plheat[p] * dt;
    }
    double pl_sum = 0.;
    for (int p = 0; p < ns; p++) pl_sum += mass[p] / rho[p] * q_plheat[p];
    plastic_work += pl_sum * dt;
  }
  // Thermal.cpp:721-748 ThermalCalcs with CalcTempInc (53-219) and
  // CalcThermalExpStrainRate (ThermalStuct.cpp:7-12)
  void thermal_calcs(double dt) {
    if (!thermal_solver) return;
    int ns = solid_part_count;
    m_maxT = 0.; m_minT = 1000.;
    for (int i = 0; i < ns; i++) {
      T[i] += dt * dTdt[i];
      if (T[i] > m_maxT) m_maxT = T[i];
      if (T[i] < m_minT) m_minT = T[i];
    }
    // Thermal.cpp:339-389 CalcConvHeat (3D): Fraser Eq. 3-121 with the contact
    // area dS^2 = (m / rho)^(2/3) of Eq. 3-119
    for (int i = 0; i < N; i++)
      if (thermal_bc[i] == 1) {
        double dS2 = std::pow(mass[i] / rho[i], 2.0 / 3.0);
        q_conv[i] = rho[i] * h_conv[i] * dS2 * (T_inf[i] - T[i]) / mass[i];
      }
    std::vector<double> tmp(N, 0.0);
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int i = 0; i < ns; i++) {
      if (is_mesh(i)) continue;
      double s = 0.;
      for (int64_t k = nb_off[i]; k < nb_off[i + 1]; ++k) {
        int j = nb_idx[k];
        int ce = grad_corr ? i : -1;
        if (j > i) s += pair_conduction(i, j, ce); else s -= pair_conduction(j, i, ce);
      }
      tmp[i] = s;
    }
    for (int i = 0; i < ns; i++) {
      double f = 1. / (rho[i] * cp_T[i]);
      dTdt[i] = f * (tmp[i] + q_conv[i] + q_source[i] + q_plheat[i] * pl_work_heat_frac + q_cont_conv[i]);
    }
    for (int i = ns; i < N; i++) dTdt[i] = 0.;
    for (int p = 0; p < N; p++) {
      double s = th_exp[p] * dTdt[p];
      for (int k = 0; k < 3; ++k) at(srate[p], k, k) = at(srate[p], k, k) + s * 1.0;
    }
  }
  // Domain.cpp:1752-1808 CalcKinEnergyEqn, 1810-1829 CalcIntEnergyEqn
  void energies() {
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int i = 0; i < N; i++) {
      double s = 0.;
      for (int64_t k = nb_off[i]; k < nb_off[i + 1]; ++k) {
        int j = nb_idx[k];
        if (j > i) s += pair_kin(i, j); else s -= pair_kin(j, i);
      }
      dkin[i] = s;
    }
    double inc = 0.;
    for (int i = 0; i < N; i++) inc += dkin[i];
    kin_energy_sum += inc * deltat;
    int mx = contact ? first_fem[0] : N;
    inc = 0.;
    for (int i = 0; i < mx; i++) {
      const M3& S = tau[i]; const M3& R = srate[i];
      dint[i] = mass[i] / rho[i] *
                (at(S, 0, 0) * at(R, 0, 0) + 2.0 * at(S, 0, 1) * at(R, 1, 0) + 2.0 * at(S, 0, 2) * at(R, 2, 0) +
                 at(S, 1, 1) * at(R, 1, 1) + 2.0 * at(S, 1, 2) * at(R, 2, 1) + at(S, 2, 2) * at(R, 2, 2));
      inc += dint[i];
    }
    int_energy_sum += inc * deltat;
  }
  // Contact_Wang.cpp:15-348 CalcContactForcesWang (solid particles in
  // ascending order, each over its contact pairs in ascending mesh index)
  void contact_wang() {
    for (int i = 0; i < N; ++i) { contforce[i] = v3(0, 0, 0); delta_cont[i] = 0.; }
    for (auto& f : m_contact_force) f = v3(0, 0, 0);
    contact_force_sum = 0.; contact_reaction_sum = 0.;
    double ext_step = 0.;
    for (int P1 = 0; P1 < N; ++P1)
      for (int64_t k = cp_off[P1]; k < cp_off[P1 + 1]; ++k) {
        int P2 = cp_idx[k];
        V3 vr = sub(v[P1], v[P2]);
        const V3& n2 = normal[P2];
        double delta_ = -dot(n2, vr);
        int m = mesh_of[P2];
        const TriMesh& M = meshes[m];
        const Element& e = M.element[elem_of[P2]];
        V3 x_pred = add(add(x[P1], scl(deltat, v[P1])), v3(a[P1].c[0] * deltat * deltat / 2.0,
                                                             a[P1].c[1] * deltat * deltat / 2.0,
                                                             a[P1].c[2] * deltat * deltat / 2.0));
        double dist = dot(n2, x_pred) - e.pplane;
        if (dist < h[P1]) {
          V3 qj = sub(x[P1], scl(dist, n2));
          bool inside = true;
          int ii = 0;
          while (ii < 3 && inside) {
            int jj = ii + 1; if (jj > 2) jj = 0;
            double crit = dot(cross(sub(M.node[e.node[jj]], M.node[e.node[ii]]), sub(qj, M.node[e.node[ii]])), n2);
            if (crit < 0.0) inside = false;
            ii++;
          }
          if (inside) {
            double delta = h[P1] - dist;
            double kij;
            if (contact_alg == 1) kij = PFAC * cont_stiff[P1];
            else if (contact_alg == 2) kij = PFAC * std::pow(mass[P1] / rho[P1], 2.0 / 3.0);
            else kij = 2.0 * mass[P1] / (deltat * deltat);
            double omega = std::sqrt(kij / mass[P1]);
            double psi_cont = 2. * mass[P1] * omega * DFAC;
            contforce[P1] = scl(kij * delta - psi_cont * delta_, n2);
            delta_cont[P1] = delta;
            a[P1] = add(a[P1], v3(contforce[P1].c[0] / mass[P1], contforce[P1].c[1] / mass[P1], contforce[P1].c[2] / mass[P1]));
            if (friction_sta > 0.) {
              V3 du = sub(sub(x_pred, x[P1]), scl(deltat, v[P2]));
              double dn = dot(du, n2);
              V3 delta_tg = sub(du, scl(dn, n2));
              V3 tgforce = scl(kij, delta_tg);
              if (norm(tgforce) < friction_sta * norm(contforce[P1])) {
                V3 q = v3(tgforce.c[0] / mass[P1], tgforce.c[1] / mass[P1], tgforce.c[2] / mass[P1]);
                contforce[P1] = sub(contforce[P1], q);
                a[P1] = sub(a[P1], q);
              } else {  // dynamic branch (Contact_Wang.cpp:284-290)
                ++dyn_friction_count;
                double s = friction_dyn * norm(contforce[P1]);
                double nt = norm(tgforce);
                V3 td = v3(s * tgforce.c[0] / nt, s * tgforce.c[1] / nt, s * tgforce.c[2] / nt);
                contforce[P1] = sub(contforce[P1], td);
                a[P1] = sub(a[P1], v3(td.c[0] / mass[P1], td.c[1] / mass[P1], td.c[2] / mass[P1]));
              }
            }
            contact_force_sum += norm(contforce[P1]);
            m_contact_force[m] = add(m_contact_force[m], contforce[P1]);
            contact_reaction_sum += dot(a[P1], n2) * mass[P1];
            ext_step += dot(contforce[P1], v[P2]);
          }
        }
      }
    ext_forces_work += ext_step * deltat;
  }
  // Contact.cpp:41-55 UpdateContactParticles
  void update_contact_particles() {
    for (size_t m = 0; m < meshes.size(); ++m) {
      TriMesh& M = meshes[m];
      for (size_t e = 0; e < M.element.size(); ++e) {
        V3 vv = v3(0, 0, 0);
        for (int en = 0; en < M.dimension; en++) vv = add(vv, M.node_v[M.element[e].node[en]]);
        int p = first_fem[m] + (int)e;
        v[p] = v3(vv.c[0] / M.dimension, vv.c[1] / M.dimension, vv.c[2] / M.dimension);
        a[p] = v3(0, 0, 0);
        normal[p] = M.element[e].normal;
      }
    }
  }

  // -------------------------------------------------------------- solver
  int prepare(double dt) {  // SolverKickDrift.cpp:23-115
    if (N == 0) return set_err(WF_ERR_STATE, "no particles");
    if (nspec > 0 && (contact || grad_corr || mode == 1))
      return set_err(WF_ERR_UNSUPPORTED, "batched specimens: no contact, gradKernelCorr or reference-structured mode");
    if (dim != 3) return set_err(WF_ERR_UNSUPPORTED, "only Dimension = 3 is supported");
    if (grad_corr && mode == 1)
      return set_err(WF_ERR_UNSUPPORTED, "kernel-gradient correction runs the locking sums (cpu_mode 0)");
    for (int i = 0; i < N; ++i) {
      if (!is_free[i]) return set_err(WF_ERR_UNSUPPORTED, "fixed (non-free) particles are not supported");
      if (pres_eq[i] != 0) return set_err(WF_ERR_UNSUPPORTED, "only PresEq = 0 is supported");
    }
    if (solid_part_count < 0) solid_part_count = N;
    if (auto_ts_cont && contact && integrator == 0)
      return set_err(WF_ERR_UNSUPPORTED,
                     "auto_ts_cont with contact: the kick-drift solver reads Domain::min_force_ts, which nothing "
                     "on its contact path sets");
    deltat = deltatint = deltatmin = dt;  // SolverKickDrift.cpp:30, SolverLeapfrog.cpp:33
    for (int i = 0; i < N; i++) pressure[i] = eos0(Cs[i], P0[i], rho[i], rho0[i]);  // InitialChecks
    int rc = cell_initiate();
    if (rc) return rc;
    if (contact) {
      for (int i = 0; i < N; i++) ID_orig[i] = ID[i];
      for (int i = 0; i < N; i++) {
        double bulk = Cs[i] * Cs[i] * rho[i];
        double dS = std::pow(mass[i] / rho[i], 0.33333);
        cont_stiff[i] = 9. * bulk * G[i] / (3. * bulk + G[i]) * dS;
      }
      rc = neighbour_search();
      if (rc) return rc;
      rc = calculate_surface(1);
      if (rc) return rc;
    }
    nb_cleared = true;  // ClearNbData
    steps = 0; isfirst = true; isyielding = false; ts_i = 0; check_nb_every_time = false;
    for (auto& q : spec) q = SpecSched();
    prev_deltat = deltat;
    prepared = true;
    return WF_OK;
  }
  int step() {  // SolverKickDrift.cpp:117-393
    int rc = begin_step();
    if (rc) return rc;
    finish_step();
    return WF_OK;
  }
  // StartAcceleration and the neighbour-search schedule (SolverKickDrift.cpp:117-186).
  int begin_step() {
    int rc;
    // StartAcceleration (Domain.cpp:1519-1597) for free particles: the
    // tensile-instability stress TIR = V diag(f(L)) V^T of Sigma with
    // f(l) = -TI l / rho^2 for l > 0, else 0 (3D branch, :1557-1569).
    for (int i = 0; i < N; i++) {
      if (TI[i] > 0.0) {
        double rho2 = rho[i] * rho[i];
        double pc = TI[i] / (rho2);
        double L[3];
        M3 V;
        eig_sym3(sigma[i], L, V);
        M3 Val = zero3();
        for (int k = 0; k < 3; ++k) at(Val, k, k) = (L[k] > 0) ? -pc * L[k] : 0.0;
        TIR[i] = matmul(matmul(V, Val), trans(V));
      }
    }
    for (int i = 0; i < N; i++) { a[i] = v3(0, 0, 0); dDensity[i] = 0.; srate[i] = zero3(); rrate[i] = zero3(); }
    double mx = 0;
    for (int i = 0; i < N; i++) if (pl_strain[i] > mx) mx = pl_strain[i];
    max_pl = mx;
    V3 md = v3(0, 0, 0);
    for (int i = 0; i < solid_part_count; i++)
      for (int j = 0; j < 3; j++) if (disp[i].c[j] * disp[i].c[j] > md.c[j]) md.c[j] = disp[i].c[j] * disp[i].c[j];
    for (int j = 0; j < 3; j++) md.c[j] = std::sqrt(md.c[j]);
    check_nb_every_time = norm(md) > 0.1 * hmax;
    if (nspec > 0) return batch_schedule();
    if (mx > MIN_PS_FOR_NBSEARCH && !isyielding) {
      nb_cleared = true;
      if ((rc = neighbour_search())) return rc;
      if (contact && (rc = contact_nb_update())) return rc;
      isyielding = true;
    }
    bool regular = false;
    if (mx > MIN_PS_FOR_NBSEARCH || isfirst || check_nb_every_time)
      if (ts_i == 0 && nb_cleared) {
        if ((rc = neighbour_search())) return rc;
        if (h_update) update_smoothing_length();  // after CalcPairPosList (SolverKickDrift.cpp:169-171)
        if (contact && (rc = contact_nb_update())) return rc;
        regular = true;
      }
    // CalcGradCorrMatrix: the kick-drift solver at its first step only
    // (SolverKickDrift.cpp:189-191); the leapfrog solver after every regular
    // search and at the first step (SolverLeapfrog.cpp:186-204).
    if (grad_corr && (isfirst || (integrator == 1 && regular))) calc_grad_corr();
    return WF_OK;
  }
  // Each specimen's rebuild decision (first yield, or its own ts_nb_inc
  // cadence while yielding, SolverKickDrift.cpp:153-186) from the largest
  // plastic strain of its own particles; one search serves every specimen that
  // asks, and the others keep their rows.
  int batch_schedule() {
    std::vector<double> mxs(nspec, 0.0);
    for (int i = 0; i < N; i++)
      if (pl_strain[i] > mxs[spec_of[i]]) mxs[spec_of[i]] = pl_strain[i];
    std::vector<char> srch(nspec, 0);
    bool any = false;
    for (int q = 0; q < nspec; ++q) {
      SpecSched& sq = spec[q];
      sq.max_pl = mxs[q];
      if (mxs[q] > MIN_PS_FOR_NBSEARCH && !sq.isyielding) {
        srch[q] = 1;
        sq.isyielding = true;
      } else if ((mxs[q] > MIN_PS_FOR_NBSEARCH || isfirst) && sq.ts_i == 0 && sq.nb_cleared) {
        srch[q] = 1;
      }
      if (srch[q]) { sq.nb_cleared = false; sq.searches++; any = true; }
    }
    if (!any) return WF_OK;
    std::vector<int64_t> off0 = nb_off;
    std::vector<int> idx0 = nb_idx;
    int rc = neighbour_search();
    if (rc) return rc;
    std::vector<int64_t> off1(N + 1, 0);
    std::vector<int> idx1;
    idx1.reserve(nb_idx.size());
    for (int i = 0; i < N; ++i) {
      bool fresh = srch[spec_of[i]] != 0;
      const std::vector<int64_t>& o = fresh ? nb_off : off0;
      const std::vector<int>& x = fresh ? nb_idx : idx0;
      for (int64_t k = o[i]; k < o[i + 1]; ++k) idx1.push_back(x[k]);
      off1[i + 1] = (int64_t)idx1.size();
      Nb[i] = (int)(off1[i + 1] - off1[i]);
    }
    nb_off.swap(off1);
    nb_idx.swap(idx1);
    return WF_OK;
  }
  // UpdateSmoothingLength (Domain.cpp:2493-2510): h -= h/3 (dDensity/Density) dt
  // within (hmin, hmax) = (h0/2, h0) (Particle.cpp:58-61).  Both solvers call
  // it after StartAcceleration has zeroed dDensity (Domain.cpp:1586), so
  // htent == h, which is never below hmax = h0 while h == h0: h stays h0.
  void update_smoothing_length() {
    for (int i = 0; i < solid_part_count; i++) {
      double htent = h[i] - h[i] * 0.33333333 * dDensity[i] / rho[i] * deltat;
      if (htent > 0.5 * hini[i] && htent < hini[i]) h[i] = htent;
    }
  }
  // CheckMinTSVel (Domain.cpp:265-299): CFL * (shortest neighbour distance) /
  // (Cs + |v|) over every particle (no neighbours: distance 1000).
  void check_min_ts_vel() {
    deltatmin = deltatint;
    for (int i = 0; i < N; i++) {
      double mn = 1000.;
      for (int64_t k = nb_off[i]; k < nb_off[i + 1]; ++k) {
        double d = norm(sub(x[nb_idx[k]], x[i]));
        if (d < mn) mn = d;
      }
      double test = CFL * mn / (Cs[i] + norm(v[i]));
      if (deltatmin > test) deltatmin = test;
    }
  }
  // CheckMinTSAccel (Domain.cpp:304-319): sqrt_h_a sqrt(h / |a|); it restarts
  // from deltatint, so with both criteria on only this one counts.
  void check_min_ts_accel() {
    deltatmin = deltatint;
    for (int i = 0; i < N; i++) {
      double test = sqrt_h_a * std::sqrt(h[i] / norm(a[i]));
      if (deltatmin > test) deltatmin = test;
    }
  }
  // AdaptiveTimeStep (Domain.cpp:206-239).  The contact term (auto_ts_cont)
  // reads min_force_ts, which the leapfrog solver sets to the initial dt
  // (SolverLeapfrog.cpp:95), never below deltat; the kick-drift solver is
  // rejected at the prologue.  The floor manual_min_ts is an int member
  // (Domain.h:328) holding 0, so it never applies.
  void adaptive_time_step() {
    if (deltatint > deltatmin) {
      if (deltat < deltatmin) deltat = 2.0 * deltat * deltatmin / (deltat + deltatmin);
      else deltat = deltatmin;
    } else {
      if (deltatint != deltat) deltat = 2.0 * deltat * deltatint / (deltat + deltatint);
      else deltat = deltatint;
    }
  }
  void time_step_control() {
    prev_deltat = deltat;
    if (auto_ts) check_min_ts_vel();
    if (auto_ts_acc) check_min_ts_accel();
    if (auto_ts || auto_ts_acc) adaptive_time_step();
  }
  // SolverFraser.cpp:212-330 (SolveDiffUpdateFraser): density and rates from
  // x(n), v(n), the stress update, then the acceleration from the new stress,
  // contact, x += v dt + a dt^2 / 2 and v += a dt.  The checker of the
  // reference's own run log of this solver (examples/input/
  // Contact_Compression.out); the library does not run this integrator.
  void fraser_body() {
    pass_density();
    for (int i = 0; i < N; i++) rho[i] += deltat * dDensity[i];
    pass_rates();
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int i = 0; i < solid_part_count; i++) if (!is_mesh(i)) stress_strain(i, deltat);
    pass_accel();
    if (contact) contact_wang();
    general_after();
    for (int i = 0; i < N; i++) {
      x_prev[i] = x[i];
      V3 du;
      for (int k = 0; k < 3; ++k) du.c[k] = v[i].c[k] * deltat + 0.5 * a[i].c[k] * deltat * deltat;
      disp[i] = add(disp[i], du);
      x[i] = add(x[i], du);
    }
    for (int i = 0; i < N; i++) v[i] = add(v[i], scl(deltat, a[i]));
    general_after();
  }
  // The rest of the step (force passes, kicks, drift, stress, thermal, bookkeeping).
  void finish_step() {
    if (integrator == 2) {
      fraser_body();
    } else {
    pass_accel();
    general_after();
    if (contact) contact_wang();
    if (integrator == 1) {
      // SolverLeapfrog.cpp:233-260: velocities at half steps; the first step
      // starts from v - a dt/2, then v += a (dt_prev + dt)/2.
      if (isfirst)
        for (int i = 0; i < N; i++) v[i] = sub(v[i], v3(a[i].c[0] * 0.5 * deltat, a[i].c[1] * 0.5 * deltat, a[i].c[2] * 0.5 * deltat));
      general_after();
      time_step_control();  // SolverLeapfrog.cpp:257-260
      for (int i = 0; i < N; i++) {
        double f = 0.5 * (prev_deltat + deltat);
        v[i] = add(v[i], v3(a[i].c[0] * f, a[i].c[1] * f, a[i].c[2] * f));
      }
      general_after();
      pass_density();  // SolverLeapfrog.cpp:263-275 (x at n, v at n+1/2)
      for (int i = 0; i < N; i++) rho[i] += deltat * dDensity[i];
      for (int i = 0; i < N; i++) {
        x_prev[i] = x[i];
        V3 du = scl(deltat, v[i]);
        disp[i] = add(disp[i], du);
        x[i] = add(x[i], du);
      }
      pass_rates();  // x at n+1, v at n+1/2 (:287-291)
    } else {
    time_step_control();  // SolverKickDrift.cpp:216-219
    for (int i = 0; i < N; i++) v[i] = add(v[i], scl(0.5 * prev_deltat, a[i]));
    general_after();
    pass_density();
    for (int i = 0; i < N; i++) rho[i] += deltat * dDensity[i];
    for (int i = 0; i < N; i++) {
      x_prev[i] = x[i];
      V3 du = scl(deltat, v[i]);
      disp[i] = add(disp[i], du);
      x[i] = add(x[i], du);
    }
    for (int i = 0; i < N; i++) v[i] = add(v[i], v3(a[i].c[0] * deltat / 2., a[i].c[1] * deltat / 2., a[i].c[2] * deltat / 2.));
    general_after();
    pass_rates();
    }
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int i = 0; i < solid_part_count; i++) if (!is_mesh(i)) stress_strain(i, deltat);
    }  // kick-drift and leapfrog bodies
    plastic_work_heat(deltat);
    thermal_calcs(deltat);
    energies();
    steps++;
    Time += deltat;
    isfirst = false;
    if (contact) {
      if (contact_mesh_auto_update) for (auto& M : meshes) M.update(deltat);
      update_contact_particles();
    }
    if (max_pl > MIN_PS_FOR_NBSEARCH) {  // max pl_strain at the start of the step
      if (ts_i == (ts_nb_inc - 1)) nb_cleared = true;  // ClearNbData
      ts_i++;
      if (ts_i > (ts_nb_inc - 1)) ts_i = 0;
    }
    for (auto& q : spec)  // each specimen's own cadence
      if (q.max_pl > MIN_PS_FOR_NBSEARCH) {
        if (q.ts_i == (ts_nb_inc - 1)) q.nb_cleared = true;
        q.ts_i++;
        if (q.ts_i > (ts_nb_inc - 1)) q.ts_i = 0;
      }
  }
};

#include "wf_tangent.inc"

// ---------------------------------------------------------------- field maps
double* f64_scalar(Domain* d, const std::string& f) {
  (void)d; (void)f; return nullptr;
}
std::vector<double>* f64_field(Domain* d, const std::string& f) {
  if (f == "G") return &d->G;
  if (f == "Cs") return &d->Cs;
  if (f == "Sigmay") return &d->sigmay;
  if (f == "Ep") return &d->Ep;
  if (f == "Alpha") return &d->alpha;
  if (f == "Beta") return &d->beta;
  if (f == "TI") return &d->TI;
  if (f == "TIInitDist") return &d->TIInitDist;
  if (f == "TIn") return &d->TIn;
  if (f == "k_T") return &d->k_T;
  if (f == "cp_T") return &d->cp_T;
  if (f == "T") return &d->T;
  if (f == "th_exp") return &d->th_exp;
  if (f == "Density") return &d->rho;
  if (f == "RefDensity") return &d->rho0;
  if (f == "Mass") return &d->mass;
  if (f == "h") return &d->h;
  if (f == "P0") return &d->P0;
  if (f == "q_source") return &d->q_source;
  if (f == "q_conv") return &d->q_conv;
  if (f == "T_inf") return &d->T_inf;
  if (f == "h_conv") return &d->h_conv;
  if (f == "Pressure") return &d->pressure;
  if (f == "pl_strain") return &d->pl_strain;
  if (f == "dTdt") return &d->dTdt;
  if (f == "eff_strain_rate") return &d->eff_strain_rate;
  if (f == "q_plheat") return &d->q_plheat;
  if (f == "delta_pl_strain") return &d->delta_pl_strain;
  if (f == "dDensity") return &d->dDensity;
  return nullptr;
}
std::vector<V3>* v3_field(Domain* d, const std::string& f) {
  if (f == "x") return &d->x;
  if (f == "v") return &d->v;
  if (f == "a") return &d->a;
  if (f == "Displacement") return &d->disp;
  if (f == "normal") return &d->normal;
  if (f == "contforce") return &d->contforce;
  return nullptr;
}
std::vector<M3>* m3_field(Domain* d, const std::string& f) {
  if (f == "Sigma") return &d->sigma;
  if (f == "ShearStress") return &d->tau;
  if (f == "StrainRate") return &d->srate;
  if (f == "RotationRate") return &d->rrate;
  if (f == "Strain") return &d->strain;
  if (f == "Strain_pl") return &d->strain_pl;
  if (f == "TIR") return &d->TIR;
  if (f == "gradCorrM") return &d->gcm;
  return nullptr;
}
std::vector<int>* i32_field(Domain* d, const std::string& f) {
  if (f == "PresEq") return &d->pres_eq;
  if (f == "Fail") return &d->fail_crit;
  if (f == "Material_model") return &d->model;
  if (f == "mat") return &d->mat;
  if (f == "Material") return &d->material_idx;
  if (f == "ID") return &d->ID;
  if (f == "IsFree") return &d->is_free;
  if (f == "Nb") return &d->Nb;
  if (f == "Thermal_BC") return &d->thermal_bc;
  return nullptr;
}

}  // namespace

// ============================================================================ C API (wfo_ prefix)
extern "C" {
struct wfo_domain;
static Domain* D(wfo_domain* p) { return reinterpret_cast<Domain*>(p); }

int wfo_version(void) { return 10000; }
const char* wfo_last_error(void) { return g_err.c_str(); }
int wfo_domain_create(int dimension, wfo_domain** out) {
  if (!out) return set_err(WF_ERR_ARG, "null out");
  if (dimension != 3) return set_err(WF_ERR_UNSUPPORTED, "only Dimension = 3 is supported");
  Domain* d = new Domain();
  d->dim = dimension;
  *out = reinterpret_cast<wfo_domain*>(d);
  return WF_OK;
}
int wfo_domain_destroy(wfo_domain* d) { delete D(d); return WF_OK; }
int wfo_set_domain_f64(wfo_domain* p, const char* name, double v) {
  Domain* d = D(p); std::string n(name ? name : "");
  if (n == "Cellfac") d->Cellfac = v;
  else if (n == "pl_work_heat_frac") d->pl_work_heat_frac = v;
  else if (n == "friction_sta") d->friction_sta = v;
  else if (n == "friction_dyn") d->friction_dyn = v;
  else if (n == "PFAC") d->PFAC = v;
  else if (n == "CFL") d->CFL = v;
  else if (n == "sqrt_h_a") d->sqrt_h_a = v;
  else if (n == "DFAC") d->DFAC = v;
  else if (n == "contact_force_factor" || n == "nb_skin") {}  // nb_skin: a GPU search strategy, same rows
  else if (n.rfind("DomMax.", 0) == 0 && n.size() == 8) d->DomMax[n[7] - 'x'] = v;
  else if (n.rfind("DomMin.", 0) == 0 && n.size() == 8) d->DomMin[n[7] - 'x'] = v;
  else return set_err(WF_ERR_ARG, "unknown domain f64 field " + n);
  return WF_OK;
}
int wfo_set_domain_i32(wfo_domain* p, const char* name, int v) {
  Domain* d = D(p); std::string n(name ? name : "");
  if (n == "ts_nb_inc") d->ts_nb_inc = v;
  else if (n == "pl_heating") d->pl_heating = v;
  else if (n == "thermal_solver") d->thermal_solver = v;
  else if (n == "contact") d->contact = v;
  else if (n == "contact_mesh_auto_update") d->contact_mesh_auto_update = v;
  else if (n == "contact_alg") d->contact_alg = v;
  else if (n == "cpu_mode") d->mode = v;
  else if (n == "integrator") d->integrator = v;
  else if (n == "gradKernelCorr") d->grad_corr = v;
  else if (n == "h_update") d->h_update = v != 0;
  else if (n == "cpu_threads" || n == "Nproc") d->nthreads = v > 0 ? v : 1;
  else if (n == "auto_ts") d->auto_ts = v != 0;
  else if (n == "auto_ts_acc") d->auto_ts_acc = v != 0;
  else if (n == "auto_ts_cont") d->auto_ts_cont = v != 0;
  else if (n == "nonlock_sum") { if (!v) return set_err(WF_ERR_UNSUPPORTED, "only the Nishimura sum is supported"); }
  else if (n == "GradientType") { if (v) return set_err(WF_ERR_UNSUPPORTED, "only GradientType 0 is supported"); }
  else if (n == "precision" || n == "device" || n == "use_graph" || n == "gather_block" || n == "gather_lanes" ||
           n == "particle_block") {}  // GPU launch shapes: no effect on the arithmetic
  else return set_err(WF_ERR_ARG, "unknown domain i32 field " + n);
  return WF_OK;
}
int wfo_get_domain_f64(wfo_domain* p, const char* name, double* v) {
  Domain* d = D(p); std::string n(name ? name : "");
  if (n == "Time") *v = d->Time;
  else if (n == "deltat") *v = d->deltat;
  else if (n == "hmax") *v = d->hmax;
  else if (n == "int_energy_sum") *v = d->int_energy_sum;
  else if (n == "kin_energy_sum") *v = d->kin_energy_sum;
  else if (n == "plastic_work") *v = d->plastic_work;
  else if (n == "contact_force_sum") *v = d->contact_force_sum;
  else if (n == "contact_reaction_sum") *v = d->contact_reaction_sum;
  else if (n == "ext_forces_work") *v = d->ext_forces_work;
  else if (n == "max_pl_strain") *v = d->max_pl;
  else if (n == "m_maxT") *v = d->m_maxT;
  else if (n == "m_minT") *v = d->m_minT;
  else if (n == "tangent_mismatch") *v = d->tangent_mismatch;
  else return set_err(WF_ERR_ARG, "unknown domain f64 read " + n);
  return WF_OK;
}
int wfo_batch_specimens(wfo_domain* p, const int64_t* first, const int64_t* count, int nspec) {
  Domain* d = D(p);
  if (nspec < 1 || !first || !count) return set_err(WF_ERR_ARG, "batch: nspec >= 1 and both arrays are required");
  std::vector<int> of(d->N, -1);
  for (int q = 0; q < nspec; ++q) {
    if (first[q] < 0 || count[q] < 1 || first[q] + count[q] > d->N) return set_err(WF_ERR_ARG, "batch: range out of bounds");
    for (int64_t i = first[q]; i < first[q] + count[q]; ++i) {
      if (of[i] >= 0) return set_err(WF_ERR_ARG, "batch: specimens overlap");
      of[i] = q;
    }
  }
  for (int v : of) if (v < 0) return set_err(WF_ERR_ARG, "batch: every particle must belong to a specimen");
  d->nspec = nspec;
  d->spec_of = of;
  d->spec_first.assign(first, first + nspec);
  d->spec_count.assign(count, count + nspec);
  d->spec.assign(nspec, Domain::SpecSched());
  return WF_OK;
}
int wfo_batch_get_i32(wfo_domain* p, int q, const char* name, int64_t* v) {
  Domain* d = D(p);
  std::string n(name ? name : "");
  if (q < 0 || q >= d->nspec) return set_err(WF_ERR_ARG, "batch: no such specimen");
  if (n == "nb_searches") *v = d->spec[q].searches;
  else if (n == "yielding") *v = d->spec[q].isyielding ? 1 : 0;
  else if (n == "first") *v = d->spec_first[q];
  else if (n == "particle_count") *v = d->spec_count[q];
  else return set_err(WF_ERR_ARG, "batch: unknown field " + n);
  return WF_OK;
}
int wfo_get_domain_i32(wfo_domain* p, const char* name, int64_t* v) {
  Domain* d = D(p); std::string n(name ? name : "");
  if (n == "particle_count") *v = d->N;
  else if (n == "solid_part_count") *v = d->solid_part_count;
  else if (n == "steps") *v = d->steps;
  else if (n == "pair_count") *v = (int64_t)d->sm_pairs.size();
  else if (n == "contact_pair_count") *v = (int64_t)d->cp_idx.size();
  else if (n == "dynamic_friction_count") *v = d->dyn_friction_count;
  else if (n == "nb_searches") *v = d->nb_searches;
  else if (n == "surface_count") *v = d->surface_count;
  else if (n == "nan_particles") *v = d->nan_count;
  else if (n.rfind("CellNo.", 0) == 0 && n.size() == 8) *v = d->CellNo[n[7] - 'x'];
  else return set_err(WF_ERR_ARG, "unknown domain i32 read " + n);
  return WF_OK;
}
int wfo_kernel_set(wfo_domain* p, int kt) {
  if (kt != 0) return set_err(WF_ERR_UNSUPPORTED, "only the cubic spline kernel (0) is supported");
  D(p)->Cellfac = 2.0;
  return WF_OK;
}
int wfo_add_box_length(wfo_domain* p, int tag, const double V[3], double Lx, double Ly, double Lz, double r,
                       double density, double h, int type, int rotation, int random, int fixed) {
  return D(p)->add_box(tag, v3(V[0], V[1], V[2]), Lx, Ly, Lz, r, density, h, type, rotation, random != 0, fixed != 0);
}
int wfo_add_cylinder_length(wfo_domain* p, int tag, const double V[3], double Rxy, double Lz, double r,
                            double density, double h, int fixed, int ghost) {
  if (ghost) return set_err(WF_ERR_UNSUPPORTED, "ghost rows are not supported");
  return D(p)->add_cylinder(tag, v3(V[0], V[1], V[2]), Rxy, Lz, r, density, h, fixed != 0);
}
int wfo_assign_zone(wfo_domain* p, const double s[3], const double e[3], int id, int64_t* count) {
  int64_t c = D(p)->assign_zone(v3(s[0], s[1], s[2]), v3(e[0], e[1], e[2]), id);
  if (count) *count = c;
  return WF_OK;
}
int wfo_set_particle_f64(wfo_domain* p, const char* field, int zone, double value) {
  Domain* d = D(p);
  auto* f = f64_field(d, field ? field : "");
  if (!f) return set_err(WF_ERR_ARG, std::string("unknown particle f64 field ") + (field ? field : ""));
  for (int i = 0; i < d->N; ++i) if (zone < 0 || d->ID[i] == zone) (*f)[i] = value;
  return WF_OK;
}
int wfo_set_particle_i32(wfo_domain* p, const char* field, int zone, int value) {
  Domain* d = D(p);
  std::string fn(field ? field : "");
  if (fn == "print_history") return WF_OK;
  auto* f = i32_field(d, fn);
  if (!f) return set_err(WF_ERR_ARG, "unknown particle i32 field " + fn);
  for (int i = 0; i < d->N; ++i) if (zone < 0 || d->ID[i] == zone) (*f)[i] = value;
  if (fn == "ID") for (int i = 0; i < d->N; ++i) if (zone < 0 || d->ID_orig[i] == zone) {}
  return WF_OK;
}
int wfo_set_particle_array_f64(wfo_domain* p, const char* field, const double* src, int64_t n) {
  Domain* d = D(p); std::string fn(field ? field : "");
  if (auto* f = f64_field(d, fn)) { if (n != d->N) return set_err(WF_ERR_ARG, "size"); for (int i = 0; i < d->N; ++i) (*f)[i] = src[i]; return WF_OK; }
  if (auto* f = v3_field(d, fn)) { if (n != 3LL * d->N) return set_err(WF_ERR_ARG, "size"); for (int i = 0; i < d->N; ++i) for (int c = 0; c < 3; ++c) (*f)[i].c[c] = src[3 * i + c]; return WF_OK; }
  if (auto* f = m3_field(d, fn)) { if (n != 9LL * d->N) return set_err(WF_ERR_ARG, "size"); for (int i = 0; i < d->N; ++i) for (int c = 0; c < 9; ++c) (*f)[i].m[c] = src[9 * i + c]; return WF_OK; }
  return set_err(WF_ERR_ARG, "unknown particle array " + fn);
}
int wfo_get_particle_array_f64(wfo_domain* p, const char* field, double* dst, int64_t n) {
  Domain* d = D(p); std::string fn(field ? field : "");
  if (auto* f = f64_field(d, fn)) { if (n != d->N) return set_err(WF_ERR_ARG, "size"); for (int i = 0; i < d->N; ++i) dst[i] = (*f)[i]; return WF_OK; }
  if (auto* f = v3_field(d, fn)) { if (n != 3LL * d->N) return set_err(WF_ERR_ARG, "size"); for (int i = 0; i < d->N; ++i) for (int c = 0; c < 3; ++c) dst[3 * i + c] = (*f)[i].c[c]; return WF_OK; }
  if (auto* f = m3_field(d, fn)) { if (n != 9LL * d->N) return set_err(WF_ERR_ARG, "size"); for (int i = 0; i < d->N; ++i) for (int c = 0; c < 9; ++c) dst[9 * i + c] = (*f)[i].m[c]; return WF_OK; }
  return set_err(WF_ERR_ARG, "unknown particle array " + fn);
}
int wfo_get_particle_array_i32(wfo_domain* p, const char* field, int32_t* dst, int64_t n) {
  Domain* d = D(p);
  auto* f = i32_field(d, field ? field : "");
  if (!f) return set_err(WF_ERR_ARG, "unknown particle i32 array");
  if (n != d->N) return set_err(WF_ERR_ARG, "size");
  for (int i = 0; i < d->N; ++i) dst[i] = (*f)[i];
  return WF_OK;
}
int wfo_set_particle_array_i32(wfo_domain* p, const char* field, const int32_t* src, int64_t n) {
  Domain* d = D(p);
  std::string fn(field ? field : "");
  if (n != d->N) return set_err(WF_ERR_ARG, "size");
  std::vector<int>* f = fn == "not_write_surf_ID" ? &d->not_write_surf : i32_field(d, fn);
  if (!f || fn == "Nb" || fn == "IsFree") return set_err(WF_ERR_ARG, "unknown settable particle i32 array " + fn);
  for (int i = 0; i < d->N; ++i) {
    (*f)[i] = src[i];
    if (fn == "ID") d->ID_orig[i] = src[i];
  }
  return WF_OK;
}
int wfo_add_material(wfo_domain* p, int model, const double* q, int np, int* mat_id) {
  Material M; M.model = model;
  if (model == 0) { if (np < 2) return set_err(WF_ERR_ARG, "bilinear needs {E, nu}"); M.E = q[0]; M.nu = q[1]; }
  else if (model == 1) {
    if (np < 5) return set_err(WF_ERR_ARG, "hollomon needs {E, nu, sy0, K, m}");
    M.E = q[0]; M.nu = q[1]; M.sy0 = q[2]; M.K = q[3]; M.m = q[4];
    M.eps0 = M.sy0 / M.E; M.eps1 = std::pow(M.sy0 / M.K, 1. / M.m);  // Material.cpp:48-57
    if (M.eps0 > M.eps1) return set_err(WF_ERR_ARG, "Hollomon material bad definition");
  } else if (model == 2) {
    if (np < 10) return set_err(WF_ERR_ARG, "johnson-cook needs {E, nu, A, B, n, C, eps_0, m, T_m, T_t}");
    M.E = q[0]; M.nu = q[1]; M.A = q[2]; M.B = q[3]; M.n = q[4]; M.C = q[5]; M.eps_0 = q[6]; M.jm = q[7]; M.T_m = q[8]; M.T_t = q[9];
  } else return set_err(WF_ERR_UNSUPPORTED, "unknown material model");
  D(p)->materials.push_back(M);
  *mat_id = (int)D(p)->materials.size() - 1;
  return WF_OK;
}
int wfo_add_amplitude(wfo_domain* p, int id, const double* t, const double* v, int n) {
  if (n < 2) return set_err(WF_ERR_ARG, "amplitude needs at least two points");
  Amplitude A; A.id = id; A.time.assign(t, t + n); A.value.assign(v, v + n);
  D(p)->amps.push_back(A);
  return WF_OK;
}
int wfo_add_velocity_bc(wfo_domain* p, int zone, const double value[3], const double value_ang[3], int value_type,
                        int amp_id, double amp_factor) {
  BC b; b.zone = zone; b.value = v3(value[0], value[1], value[2]);
  b.value_ang = value_ang ? v3(value_ang[0], value_ang[1], value_ang[2]) : v3(0, 0, 0);
  b.value_type = value_type; b.amp_id = amp_id; b.amp_factor = amp_factor;
  D(p)->bcs.push_back(b);
  return WF_OK;
}
int wfo_add_rigid_plane(wfo_domain* p, int axis, int posit, const double p1[3], const double p2[3], int dens,
                        double hfac, int zone_id, int* mesh_id) {
  if (dens <= 0 || axis < 0 || axis > 2) return set_err(WF_ERR_ARG, "bad plane arguments");
  if (zone_id == 1) return set_err(WF_ERR_ARG, "zone id 1 marks the free surface (CalculateSurface(1))");
  int m = D(p)->add_plane(axis, posit != 0, v3(p1[0], p1[1], p1[2]), v3(p2[0], p2[1], p2[2]), dens, hfac, zone_id);
  if (mesh_id) *mesh_id = m;
  return WF_OK;
}
int wfo_set_mesh_velocity(wfo_domain* p, int mesh, const double v[3], const double w[3]) {
  Domain* d = D(p);
  if (mesh < 0 || mesh >= (int)d->meshes.size()) return set_err(WF_ERR_ARG, "mesh index");
  d->meshes[mesh].m_v = v3(v[0], v[1], v[2]);
  if (w) d->meshes[mesh].m_w = v3(w[0], w[1], w[2]);
  return WF_OK;
}
int wfo_get_contact_force(wfo_domain* p, int mesh, double out[3]) {
  Domain* d = D(p);
  if (mesh < 0 || mesh >= (int)d->m_contact_force.size()) return set_err(WF_ERR_ARG, "mesh index");
  for (int c = 0; c < 3; ++c) out[c] = d->m_contact_force[mesh].c[c];
  return WF_OK;
}
int wfo_prepare_kickdrift(wfo_domain* p, double dt) { return D(p)->prepare(dt); }
int wfo_step(wfo_domain* p, int64_t n) {
  Domain* d = D(p);
  if (!d->prepared) return set_err(WF_ERR_STATE, "wfo_step before wfo_prepare_kickdrift");
  for (int64_t s = 0; s < n; ++s) { int rc = d->step(); if (rc) return rc; }
  return WF_OK;
}
int wfo_solve_kickdrift(wfo_domain* p, double tf, double dt, double dtOut, int64_t maxidx) {
  Domain* d = D(p);
  int rc;
  if (!d->prepared && (rc = d->prepare(dt))) return rc;
  int64_t idx_out = 1;
  double tout = d->Time;
  while (d->Time <= tf && idx_out <= maxidx) {
    if ((rc = d->step())) return rc;
    if (d->Time >= tout) { idx_out++; tout += dtOut; }
  }
  return WF_OK;
}
// Domain::SolveDiffUpdateLeapFrog (SolverLeapfrog.cpp:24-451): the same
// prologue and schedule as the kick-drift loop with the leapfrog update.
int wfo_solve_leapfrog(wfo_domain* p, double tf, double dt, double dtOut, int64_t maxidx) {
  Domain* d = D(p);
  if (d->prepared && d->integrator != 1) return set_err(WF_ERR_STATE, "the domain was prepared for kick-drift");
  d->integrator = 1;
  return wfo_solve_kickdrift(p, tf, dt, dtOut, maxidx);
}
int wfo_neighbour_search(wfo_domain* p) { return D(p)->neighbour_search(); }
int wfo_get_neighbours(wfo_domain* p, int64_t* off, int32_t* idx, int64_t cap) {
  Domain* d = D(p);
  if ((int64_t)d->nb_off.size() != d->N + 1) return set_err(WF_ERR_STATE, "no neighbour list yet");
  for (int i = 0; i <= d->N; ++i) off[i] = d->nb_off[i];
  if (idx) {
    if (cap < (int64_t)d->nb_idx.size()) return set_err(WF_ERR_ARG, "idx capacity");
    for (size_t k = 0; k < d->nb_idx.size(); ++k) idx[k] = d->nb_idx[k];
  }
  return WF_OK;
}
int wfo_get_contact_pairs(wfo_domain* p, int64_t* off, int32_t* idx, int64_t cap) {
  Domain* d = D(p);
  if ((int64_t)d->cp_off.size() != d->N + 1) { for (int i = 0; i <= d->N; ++i) off[i] = 0; return WF_OK; }
  for (int i = 0; i <= d->N; ++i) off[i] = d->cp_off[i];
  if (idx) {
    if (cap < (int64_t)d->cp_idx.size()) return set_err(WF_ERR_ARG, "idx capacity");
    for (size_t k = 0; k < d->cp_idx.size(); ++k) idx[k] = d->cp_idx[k];
  }
  return WF_OK;
}
int wfo_synchronize(wfo_domain*) { return WF_OK; }
// The oracle reads at once; the asynchronous form is the same read.
int wfo_get_particle_array_f64_async(wfo_domain* p, const char* field, double* dst, int64_t n) {
  return wfo_get_particle_array_f64(p, field, dst, n);
}
// Checkpoints of the whole oracle state (a copy of the Domain object).
static std::vector<Domain*> g_slots[1];
int wfo_checkpoint_save(wfo_domain* p, int slot) {
  if (slot < 0 || slot > 15) return set_err(WF_ERR_ARG, "slot");
  auto& v = g_slots[0];
  if ((int)v.size() <= slot) v.resize(slot + 1, nullptr);
  delete v[slot];
  v[slot] = new Domain(*D(p));
  return WF_OK;
}
int wfo_checkpoint_restore(wfo_domain* p, int slot) {
  auto& v = g_slots[0];
  if (slot < 0 || slot >= (int)v.size() || !v[slot]) return set_err(WF_ERR_STATE, "checkpoint slot is empty");
  *D(p) = *v[slot];
  return WF_OK;
}
int wfo_checkpoint_free(wfo_domain*, int slot) {
  auto& v = g_slots[0];
  if (slot >= 0 && slot < (int)v.size()) { delete v[slot]; v[slot] = nullptr; }
  return WF_OK;
}
int wfo_autotune(wfo_domain*, int, int* block) { if (block) *block = 0; return WF_OK; }
// The gradient of the reaction-force loss by the FP64 tangent-linear run
// (forward mode, one dual direction per parameter) in canonical mode: the
// reference against which the GPU's reverse-mode adjoint is checked.  Same
// arguments and loss as the library's entry point; checkpoint_every has no
// effect (forward mode needs no recompute); adj_ms is 0.
int wfo_adjoint_reaction_loss(wfo_domain* p, int64_t steps, int every, int mesh, int axis, const double* target,
                              int64_t ntarget, int checkpoint_every, double* loss, double* grad, double* curve,
                              double* fwd_ms, double* adj_ms) {
  Domain* d = D(p);
  (void)checkpoint_every;
  if (!d->prepared) return set_err(WF_ERR_STATE, "adjoint before wf_prepare_kickdrift");
  if (d->mode != 0) return set_err(WF_ERR_UNSUPPORTED, "the tangent run needs cpu_mode 0");
  if (d->integrator != 0) return set_err(WF_ERR_UNSUPPORTED, "the adjoint differentiates the kick-drift step");
  if (d->grad_corr) return set_err(WF_ERR_UNSUPPORTED, "adjoint: kernel-gradient correction is not supported");
  if (d->auto_ts || d->auto_ts_acc) return set_err(WF_ERR_UNSUPPORTED, "adjoint: the time step must be fixed");
  if (!d->contact || mesh < 0 || mesh >= (int)d->meshes.size())
    return set_err(WF_ERR_ARG, "the reaction-force loss needs a rigid mesh");
  if (axis < 0 || axis > 2 || every < 1 || steps < 1 || ntarget < 1 || ntarget * every > steps || !target || !loss ||
      !grad)
    return set_err(WF_ERR_ARG, "adjoint: bad steps / sampling / target arguments");
  for (int i = 0; i < d->N; ++i) {
    if (d->Ep[i] < 0.0) return set_err(WF_ERR_UNSUPPORTED, "adjoint: particles with Ep < 0 are not supported");
    if (d->TI[i] > 0.0) return set_err(WF_ERR_UNSUPPORTED, "adjoint: tensile instability (TI > 0) is not supported");
  }
  auto t0 = std::chrono::steady_clock::now();
  Tangent T(*d);
  T.init();
  double L = 0.0;
  for (int k = 0; k < NPAR; ++k) grad[k] = 0.0;
  for (int64_t st = 0; st < steps; ++st) {
    int rc = d->begin_step();
    if (rc) return rc;
    T.step();
    d->finish_step();
    if ((st + 1) % every == 0 && (st + 1) / every <= ntarget) {
      int64_t s = (st + 1) / every - 1;
      const Dd& F = T.mcf[mesh].c[axis];
      double r = F.v - target[s];
      L += r * r;
      for (int k = 0; k < NPAR; ++k) grad[k] += 2.0 * r / (double)ntarget * F.d[k];
      if (curve) curve[s] = F.v;
    }
    T.sync();
  }
  *loss = L / (double)ntarget;
  d->tangent_mismatch = T.mismatch;
  if (fwd_ms) *fwd_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (adj_ms) *adj_ms = 0.0;
  return WF_OK;
}
int wfo_step_timed(wfo_domain* p, int64_t n, double* ms, int64_t* launches) {
  auto t0 = std::chrono::steady_clock::now();
  int rc = wfo_step(p, n);
  auto t1 = std::chrono::steady_clock::now();
  *ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  if (launches) *launches = 0;
  return rc;
}
int wfo_profile_steps(wfo_domain*, int64_t, char*, int, double*, int64_t*, int, int* nk) { *nk = 0; return WF_OK; }
// Reference-mode helper for the CPU baseline: wall time of nsteps in seconds.
double wfo_time_steps(wfo_domain* p, int64_t nsteps) {
  auto t0 = std::chrono::steady_clock::now();
  int rc = wfo_step(p, nsteps);
  auto t1 = std::chrono::steady_clock::now();
  if (rc) return -1.0;
  return std::chrono::duration<double>(t1 - t0).count();
}
}  // extern "C"
