// Host side of the GB300 kick-drift SPH library: the SPH::Domain façade
// (Source/Domain.h:113-537) over the C ABI declared in include/weldform_gb300.h.
//
// Before the solver prologue the domain is a host-side particle set in the
// reference's insertion order (generators, zones, per-particle fields).  The
// prologue uploads it into the device arena, builds the cell grid
// (CellInitiate, Neighbour.cpp:10-139) and from then on all state lives in
// HBM in cell-sorted order; host transfers map through the original index.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <map>
#include <mutex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/weldform_gb300.h"
#include "wf_adjoint.cuh"
#include "wf_device.cuh"
#include "wf_launch.h"

namespace {

thread_local std::string g_err;
int set_err(int code, const std::string& m) { g_err = m; return code; }

}  // namespace

namespace wf {
void set_last_error(const std::string& msg) { g_err = msg; }
}  // namespace wf

namespace {

struct CudaError { int code; std::string msg; };
#define CK(call)                                                                                    \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) throw CudaError{WF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)}; \
  } while (0)

const double PI = 3.14159265358979323846;

struct Vec { double c[3]; };
inline Vec vec(double a, double b, double c) { return Vec{{a, b, c}}; }

struct HostMaterial { int model; std::vector<double> p; wf::MaterialDev dev; };
struct HostAmp { int id; std::vector<double> t, v; };
struct HostBC { int zone; double value[3], ang[3]; int vt, amp; double fac; };
struct HostMesh {
  std::vector<Vec> node;
  std::vector<int> en;          // 3 per element
  std::vector<Vec> centroid, normal;
  std::vector<double> pplane, radius;
  int id = 0, first = 0;
  Vec mv = vec(0, 0, 0), mw = vec(0, 0, 0);
};

// Particle field table: name -> host vector (original order).
struct HostParticles {
  std::vector<double> f[wf::NF64_PERSIST];
  std::vector<int> i[wf::NI32_PERSIST];
  int N = 0;
};

int col_f64(const std::string& n, int* ncomp) {
  using namespace wf;
  struct E { const char* n; int c, k; };
  static const E tab[] = {
      {"x", C_X, 3}, {"v", C_V, 3}, {"a", C_A, 3}, {"Displacement", C_DISP, 3}, {"normal", C_NORMAL, 3},
      {"contforce", C_CF, 3}, {"Density", C_RHO, 1}, {"RefDensity", C_RHO0, 1}, {"Mass", C_MASS, 1}, {"h", C_H, 1},
      {"Cs", C_CS, 1}, {"P0", C_P0, 1}, {"G", C_G, 1}, {"Pressure", C_P, 1}, {"pl_strain", C_PLS, 1},
      {"delta_pl_strain", C_DPLS, 1}, {"Sigmay", C_SY, 1}, {"Ep", C_EP, 1}, {"eff_strain_rate", C_ESR, 1},
      {"T", C_T, 1}, {"dTdt", C_DTDT, 1}, {"k_T", C_KT, 1}, {"cp_T", C_CPT, 1}, {"th_exp", C_THEXP, 1},
      {"q_plheat", C_QPL, 1}, {"q_source", C_QSRC, 1}, {"Alpha", C_ALPHA, 1}, {"Beta", C_BETA, 1},
      {"ps_energy", C_PSEN, 1}, {"delta_cont", C_DCONT, 1}, {"dkin_energy_dt", C_DKIN, 1},
      {"dint_energy_dt", C_DINT, 1}, {"dDensity", C_DRHO, 1}, {"TI", C_TI, 1}, {"TIn", C_TIN, 1},
      {"TIInitDist", C_TIDIST, 1}, {"TIR", C_TIR, 6}, {"gradCorrM", C_GCM, 9}, {"Sigma", C_SIG, 6}, {"ShearStress", C_TAU, 6},
      {"Strain", C_EPS, 6}, {"Strain_pl", C_EPL, 6}, {"Strain_pl_incr", C_EPLI, 6}, {"StrainRate", C_SR, 6},
      {"RotationRate", C_RR, 3}, {"T_inf", C_TINF, 1}, {"h_conv", C_HCONV, 1}, {"q_conv", C_QCONV, 1}};
  for (const E& e : tab)
    if (n == e.n) { *ncomp = e.k; return e.c; }
  return -1;
}
int col_i32(const std::string& n) {
  using namespace wf;
  if (n == "ID") return I_ID;
  if (n == "mat") return I_MAT;
  if (n == "Material_model") return I_MODEL;
  if (n == "Fail") return I_FAIL;
  if (n == "Material") return I_MATERIAL;
  if (n == "Nb") return I_NB;
  if (n == "Thermal_BC") return I_THBC;
  return -1;
}
// Fields that exist in the reference but are fixed in this build's scope.
bool fixed_i32(const std::string& n, int v, std::string* why) {
  if (n == "PresEq") { if (v != 0) { *why = "only PresEq = 0 is supported"; return false; } return true; }
  if (n == "IsFree") { if (v != 1) { *why = "fixed (non-free) particles are not supported"; return false; } return true; }
  if (n == "print_history") return true;
  *why = "unknown particle i32 field " + n;
  return false;
}

// Morton code of a cell (10 bits per axis, interleaved).
uint64_t spread3(uint64_t v) {
  v &= 0x1fffff;
  v = (v | v << 32) & 0x1f00000000ffffULL;
  v = (v | v << 16) & 0x1f0000ff0000ffULL;
  v = (v | v << 8) & 0x100f00f00f00f00fULL;
  v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
  v = (v | v << 2) & 0x1249249249249249ULL;
  return v;
}

}  // namespace

struct wf_domain {
  int dim = 3;
  // Domain defaults (Source/Domain.cpp:78-175)
  double Cellfac = 2.0, pl_work_heat_frac = 0.9, friction_sta = 0.0, friction_dyn = 0.0, PFAC = 0.0, DFAC = 0.0;
  double DomMax[3] = {-100000000000.0, -100000000000.0, -100000000000.0};
  double DomMin[3] = {100000000000.0, 100000000000.0, 100000000000.0};
  int freeze_nb = 0;  // search only at the first step (finite-difference checks of the adjoint)
  int nan_check = 0;  // raise WF_ERR_NAN on a non-finite position at a search or non-finite energy sums
  double nb_skin = 0.1;  // Verlet skin of the search reuse, relative to the largest pair radius (0: off)
  // batched specimens (wf_batch_specimens): [first, first + count) in original order
  std::vector<int64_t> spec_first, spec_count;
  int ts_nb_inc = 5, pl_heating = 0, thermal_solver = 0, contact = 0, contact_mesh_auto_update = 1, contact_alg = 0;
  int precision = WF_PRECISION_FP64, use_graph = 1, device = 0;
  int integrator = 0;  // 0 kick-drift, 1 leapfrog
  int grad_corr = 0;   // Domain::gradKernelCorr
  int solid_part_count = -1;

  HostParticles hp;
  std::vector<HostMaterial> mats;
  std::vector<HostAmp> amps;
  std::vector<HostBC> bcs;
  std::vector<HostMesh> meshes;

  // device
  bool prepared = false;
  cudaStream_t stream = nullptr;
  wf::DevPtrs P{};
  wf::DomainConst K{};
  double* d_f = nullptr;
  int* d_i = nullptr;
  double* d_fscratch = nullptr;
  int* d_iscratch = nullptr;
  std::vector<void*> allocs;
  cudaGraphExec_t graph = nullptr;
  int graph_precision = -1;
  int graph_block = -1;
  bool h_update = false;  // accepted; no effect in these solvers (see "h_update" in the setter)
  // adaptive time step (Domain.cpp:107-170 defaults)
  int auto_ts = 0, auto_ts_acc = 0, auto_ts_cont = 0;
  double CFL = 0.7, sqrt_h_a = 0.0025;
  int gblock = 0;    // mixed gathers' threads per block (0: chosen by particle count)
  int glanes = 0;    // lanes per particle of the mixed acceleration gather (1, 2, 4, 8; 0: by particle count)
  int pblock = 0;    // per-particle kernels' threads per block (0: chosen by particle count)
  int fuse_rs = 1;   // mixed form: rate gather and stress update fused in one kernel (one lane per particle)
  // Shared-memory staging of the mixed acceleration gather: the halo lists
  // are allocated at the prologue when it is on; stage_cap is each block's
  // halo capacity (STAGE_B particles per block, 80 B of shared memory per slot).
  bool stage = false;
  int stage_cap = 896;
  bool stage_ready = false;
  // Block sizes by particle count: below ~4 blocks of 256 per SM the per-particle
  // kernels (one thread per particle, FP64 or gather latency bound) leave SMs
  // idle, so smaller blocks spread the particles over every SM.
  static int auto_block(long long n) { return n < 78000 ? 64 : (n < 156000 ? 128 : 256); }
  int gblock_now() const { return gblock ? gblock : auto_block(hp.N); }
  // Below ~60k particles a gather's time is its rows' chain of dependent
  // loads (one thread walks ~55 entries), not throughput: splitting each
  // row over lanes shortens the chain (measured on GB300, mixed step:
  // 8,004 particles best with 8 lanes, 29,520 with 4, 44,880 with 2 (135
  // against 142 us), 79,856 and up with 1).
  static int auto_lanes(long long n) { return n < 20000 ? 8 : (n < 40000 ? 4 : (n < 64000 ? 2 : 1)); }
  int glanes_now() const { return glanes ? glanes : auto_lanes(hp.N); }
  int pblock_now() const { return pblock ? pblock : auto_block(hp.N); }
  int graph_key() const {
    return (((gblock_now() * 1024 + pblock_now()) * 16 + glanes_now()) * 2 + (stage_ready && stage ? 1 : 0)) * 2 +
           (fuse_rs ? 1 : 0);
  }
  struct Region { void* p; size_t bytes; };
  std::vector<Region> regions;           // every mutable device region of the state
  std::vector<std::vector<void*>> slots; // checkpoint copies, one vector per slot
  bool shadows_valid = false;  // float shadows of the mixed form match the FP64 state
  long long launches_per_step = 0;     // launches every replay of the step graph makes
  long long search_launches = 0;       // launches in its conditional search body (0: gated form)
  // Search in a graph conditional node (opt-in "search_conditional"): fewer
  // launches on steps without a search, but ncu does not profile the kernel
  // nodes of a graph that holds conditional nodes, so the gated form is the
  // default.  Cleared when the capture fails on this device or driver.
  bool cond_ok = false;
  cudaStream_t body_stream = nullptr;  // captures the conditional search body
  // Asynchronous read-back (wf_get_particle_array_f64_async): the field is
  // gathered on the domain's stream into a snapshot buffer, and the copy to
  // the host runs on copy_stream, so steps enqueued after it overlap the copy.
  cudaStream_t copy_stream = nullptr;
  struct Snapshot {
    double* buf = nullptr;
    size_t bytes = 0;
    cudaEvent_t ready = nullptr, done = nullptr;  // gathered; copied out
    bool used = false;
  };
  std::vector<Snapshot> snaps = std::vector<Snapshot>(4);  // a ring: four reads in flight
  size_t snap_next = 0;
  // wf::SearchCond for one capture: the IF node on a fresh handle of the
  // capturing graph, its body captured on body_stream.
  struct CondCapture : wf::SearchCond {
    cudaStream_t body;
    cudaGraph_t body_graph = nullptr;
    cudaGraphConditionalHandle handle = 0;
    long long l0 = 0, body_launches = 0;
    explicit CondCapture(cudaStream_t b) : body(b) {}
    unsigned long long begin(cudaStream_t s) override {
      cudaStreamCaptureStatus st;
      cudaGraph_t g;
      const cudaGraphNode_t* deps;
      size_t nd;
      CK(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &nd));
      if (st != cudaStreamCaptureStatusActive) throw CudaError{WF_ERR_CUDA, "conditional search outside a capture"};
      CK(cudaGraphConditionalHandleCreate(&handle, g, 0, cudaGraphCondAssignDefault));
      return (unsigned long long)handle;
    }
    cudaStream_t open_body(cudaStream_t s) override {
      cudaStreamCaptureStatus st;
      cudaGraph_t g;
      const cudaGraphNode_t* deps;
      size_t nd;
      CK(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &nd));
      cudaGraphNodeParams cp = {};
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = handle;
      cp.conditional.type = cudaGraphCondTypeIf;
      cp.conditional.size = 1;
      cudaGraphNode_t node;
      CK(cudaGraphAddNode(&node, g, deps, nullptr, nd, &cp));
      body_graph = cp.conditional.phGraph_out[0];
      CK(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
      CK(cudaStreamBeginCaptureToGraph(body, body_graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
      l0 = wf::g_launches;
      return body;
    }
    void close_body() override {
      body_launches = wf::g_launches - l0;
      CK(cudaStreamEndCapture(body, &body_graph));
    }
  };
  // Ends any capture left open on the domain's streams after a failure.
  void abort_capture() {
    for (cudaStream_t st : {body_stream, stream}) {
      if (!st) continue;
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(st, &g);
        if (g) cudaGraphDestroy(g);
      }
    }
    cudaGetLastError();
  }
  // Captures one step into the step graph: with the search in a conditional
  // node when that works on this device and driver, else in the gated form.
  void capture_step_graph() {
    if (graph) { cudaGraphExecDestroy(graph); graph = nullptr; }
    graph_block = graph_key();
    for (int attempt = cond_ok ? 0 : 1; attempt < 2; ++attempt) {
      const bool cond = attempt == 0;
      try {
        if (cond && !body_stream) CK(cudaStreamCreateWithFlags(&body_stream, cudaStreamNonBlocking));
        CondCapture cc(body_stream);
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        long long l0 = wf::g_launches;
        wf::g_search_cond = cond ? &cc : nullptr;
        try {
          launch_one_step();
        } catch (...) {
          wf::g_search_cond = nullptr;
          throw;
        }
        wf::g_search_cond = nullptr;
        search_launches = cond ? cc.body_launches : 0;
        launches_per_step = wf::g_launches - l0 - search_launches;
        CK(cudaStreamEndCapture(stream, &g));
        cudaError_t e = cudaGraphInstantiate(&graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) throw CudaError{WF_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e)};
        graph_precision = precision;
        return;
      } catch (CudaError&) {
        abort_capture();
        if (graph) { cudaGraphExecDestroy(graph); graph = nullptr; }
        if (!cond) throw;
        cond_ok = false;  // capture the gated form from now on
      }
    }
  }
  double hmax = 0;
  double BLPF[3] = {0, 0, 0}, TRPR[3] = {0, 0, 0};
  int CellNo[3] = {0, 0, 0};

  ~wf_domain() { release(); }
  void release() {
    for (auto& sl : slots)
      for (void* p : sl) cudaFree(p);
    slots.clear();
    if (graph) { cudaGraphExecDestroy(graph); graph = nullptr; }
    for (void* p : allocs) cudaFree(p);
    allocs.clear();
    if (body_stream) { cudaStreamDestroy(body_stream); body_stream = nullptr; }
    if (copy_stream) { cudaStreamSynchronize(copy_stream); cudaStreamDestroy(copy_stream); copy_stream = nullptr; }
    for (auto& sn : snaps) {
      if (sn.buf) cudaFree(sn.buf);
      if (sn.ready) cudaEventDestroy(sn.ready);
      if (sn.done) cudaEventDestroy(sn.done);
      sn = Snapshot();
    }
    if (stream) { cudaStreamDestroy(stream); stream = nullptr; }
    prepared = false;
  }
  template <class T> T* dalloc(size_t n) {
    void* p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc(&p, n * sizeof(T));
    if (e != cudaSuccess) throw CudaError{WF_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e)};
    allocs.push_back(p);
    return (T*)p;
  }

  // ------------------------------------------------------------ particles
  void push(int tag, Vec x, double m0, double dens, double h, int kind) {
    using namespace wf;
    for (int c = 0; c < NF64_PERSIST; ++c) hp.f[c].push_back(0.0);
    for (int c = 0; c < NI32_PERSIST; ++c) hp.i[c].push_back(0);
    int p = hp.N++;
    for (int d = 0; d < 3; ++d) hp.f[C_X + d][p] = x.c[d];
    hp.f[C_RHO][p] = dens; hp.f[C_RHO0][p] = dens; hp.f[C_MASS][p] = m0; hp.f[C_H][p] = h;
    hp.i[I_ID][p] = tag; hp.i[I_IDORIG][p] = tag; hp.i[I_MAT][p] = -1; hp.i[I_KIND][p] = kind;
    hp.i[I_ELEM][p] = -1; hp.i[I_MESH][p] = -1; hp.i[I_ORIG][p] = p;
    hp.f[C_TIN][p] = 4.0;  // Particle.cpp:47
    hp.f[C_GCM][p] = hp.f[C_GCM + 4][p] = hp.f[C_GCM + 8][p] = 1.0;  // gradCorrM = I
  }
  double& F(int c, int p) { return hp.f[c][p]; }

  // Domain::AddCylinderLength, Source/Domain.cpp:708-860 (3D, no ghost rows).
  static int half_part_count(double r, double R, int xinc) {  // calcHalfPartCount, Domain.cpp:674-689
    int count = -1;
    if (xinc > 0) {
      count = 1;
      double yp = r;
      double xp = r + (double)(xinc - 1) * 2. * r;
      double rad = std::sqrt(yp * yp + xp * xp);
      while (rad <= R - r) {
        yp += 2. * r;
        rad = std::sqrt(yp * yp + xp * xp);
        count++;
      }
      count -= 1;
    }
    return count;
  }
  void add_cylinder(int tag, const double V[3], double Rxy, double Lz, double r, double dens, double h) {
    int nxy = half_part_count(r, Rxy, 1);
    for (double zp = V[2] + r; zp <= (V[2] + Lz - r); zp += 2. * r) {
      double yp = V[1] - r - (2. * r * (nxy - 1));
      int yinc = nxy, ysign = -1;
      for (int j = 0; j < 2 * nxy; j++) {
        int nx = half_part_count(r, Rxy, yinc);
        double xp = V[0] - r - (2. * r * (nx - 1));
        for (int i = 0; i < 2 * nx; i++) {
          push(tag, vec(xp, yp, zp), 0.0, dens, h, 0);
          xp += 2. * r;
        }
        yp += 2. * r;
        yinc += ysign;
        if (yinc < 1) { yinc = 1; ysign = 1; }
      }
    }
    solid_part_count = hp.N;
    double Mass = PI * Rxy * Rxy * Lz * dens / hp.N;
    for (int p = 0; p < hp.N; ++p) F(wf::C_MASS, p) = Mass;
  }
  // Domain::AddBoxLength, Source/Domain.cpp:326-599 (3D packings).
  void add_box(int tag, const double V[3], double Lx, double Ly, double Lz, double r, double dens, double h, int type,
               bool random) {
    int first = hp.N;
    const double qin = 0.03;
    srand(100);
    auto emit = [&](double x, double y, double z) {
      if (random) {
        double a = qin * r * double(rand()) / RAND_MAX;
        double b = qin * r * double(rand()) / RAND_MAX;
        double c = qin * r * double(rand()) / RAND_MAX;
        push(tag, vec(x + a, y + b, z + c), 0.0, dens, h, 0);
      } else {
        push(tag, vec(x, y, z), 0.0, dens, h, 0);
      }
    };
    if (type == 0) {  // hexagonal close packing
      size_t k = 0;
      double zp = V[2];
      while (zp <= (V[2] + Lz - r)) {
        size_t j = 0;
        double yp = V[1];
        while (yp <= (V[1] + Ly - r)) {
          size_t i = 0;
          double xp = V[0];
          while (xp <= (V[0] + Lx - r)) {
            double x;
            if ((k % 2 != 0) && (j % 2 != 0)) x = V[0] + (2 * i + (j % 2) + (k % 2) - 1) * r;
            else x = V[0] + (2 * i + (j % 2) + (k % 2) + 1) * r;
            double y = V[1] + (std::sqrt(3.0) * (j + (1.0 / 3.0) * (k % 2)) + 1) * r;
            double z = V[2] + ((2 * std::sqrt(6.0) / 3) * k + 1) * r;
            emit(x, y, z);
            i++;
            if ((k % 2 != 0) && (j % 2 != 0)) xp = V[0] + (2 * i + (j % 2) + (k % 2) - 1) * r;
            else xp = V[0] + (2 * i + (j % 2) + (k % 2) + 1) * r;
          }
          j++;
          yp = V[1] + (std::sqrt(3.0) * (j + (1.0 / 3.0) * (k % 2)) + 1) * r;
        }
        k++;
        zp = V[2] + ((2 * std::sqrt(6.0) / 3) * k + 1) * r;
      }
    } else {  // cubic packing
      size_t k = 0;
      double zp = V[2];
      while (zp <= (V[2] + Lz - r)) {
        size_t j = 0;
        double yp = V[1];
        while (yp <= (V[1] + Ly - r)) {
          size_t i = 0;
          double xp = V[0];
          while (xp <= (V[0] + Lx - r)) {
            emit(V[0] + (2.0 * i + 1) * r, V[1] + (2.0 * j + 1) * r, V[2] + (2.0 * k + 1) * r);
            i++;
            xp = V[0] + (2 * i + 1) * r;
          }
          j++;
          yp = V[1] + (2.0 * j + 1) * r;
        }
        k++;
        zp = V[2] + (2.0 * k + 1) * r;
      }
    }
    double mx[3] = {V[0], V[1], V[2]};
    for (int p = first; p < hp.N; ++p)
      for (int d = 0; d < 3; ++d) mx[d] = std::max(mx[d], F(wf::C_X + d, p));
    double t[3];
    for (int d = 0; d < 3; ++d) t[d] = (mx[d] + r) - V[d];
    double Mass = t[0] * t[1] * t[2] * dens / (hp.N - first);
    for (int p = 0; p < hp.N; ++p) F(wf::C_MASS, p) = Mass;  // every particle, as Domain.cpp:461-469
    solid_part_count = hp.N;
  }
  // TriMesh::AxisPlaneMesh (Mesh.cpp:82-203), CalcSpheres (:206-220) and
  // Domain::AddTrimeshParticles (Contact.cpp:10-38).
  int add_plane(int axis, bool posit, const double p1[3], const double p2[3], int dens, double hfac, int zone) {
    HostMesh M;
    int dir[3];
    if (axis == 0) { dir[0] = 1; dir[1] = 2; } else if (axis == 1) { dir[0] = 0; dir[1] = 2; } else { dir[0] = 0; dir[1] = 1; }
    dir[2] = axis;
    double dl = (p2[dir[0]] - p1[dir[0]]) / dens;
    double x2 = p1[dir[1]];
    for (int j = 0; j < dens + 1; j++) {
      double x1 = p1[dir[0]];
      for (int i = 0; i < dens + 1; i++) {
        Vec q; q.c[dir[0]] = x1; q.c[dir[1]] = x2; q.c[dir[2]] = p1[dir[2]];
        M.node.push_back(q);
        x1 += dl;
      }
      x2 += dl;
    }
    for (int j = 0; j < dens; j++)
      for (int i = 0; i < dens; i++) {
        int n0 = (dens + 1) * j + i, n1 = n0 + 1, n2 = (dens + 1) * (j + 1) + i, n3 = n2 + 1;
        int tri[2][3] = {{n0, n1, n2}, {n1, n3, n2}};
        if (!posit) { tri[0][1] = n2; tri[0][2] = n1; tri[1][0] = n1; tri[1][1] = n2; tri[1][2] = n3; }
        for (int e = 0; e < 2; ++e) {
          for (int k = 0; k < 3; ++k) M.en.push_back(tri[e][k]);
          Vec s;
          for (int d = 0; d < 3; ++d) s.c[d] = (M.node[tri[e][0]].c[d] + M.node[tri[e][1]].c[d] + M.node[tri[e][2]].c[d]) / 3.;
          M.centroid.push_back(s);
        }
      }
    int ne = (int)M.centroid.size();
    for (int e = 0; e < ne; ++e) {  // CalcNormals
      const Vec& a = M.node[M.en[3 * e]]; const Vec& b = M.node[M.en[3 * e + 1]]; const Vec& c = M.node[M.en[3 * e + 2]];
      double u[3], w[3];
      for (int d = 0; d < 3; ++d) { u[d] = b.c[d] - a.c[d]; w[d] = c.c[d] - a.c[d]; }
      double cr[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
      double ln = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
      Vec n = vec(cr[0] / ln, cr[1] / ln, cr[2] / ln);
      if (posit) n = vec(-n.c[0], -n.c[1], -n.c[2]);
      M.normal.push_back(n);
    }
    for (int e = 0; e < ne; ++e) {  // CalcSpheres: radius = farthest node; plane through the last node
      double mx = 0.;
      for (int k = 0; k < 3; ++k) {
        const Vec& q = M.node[M.en[3 * e + k]];
        double r2[3] = {q.c[0] - M.centroid[e].c[0], q.c[1] - M.centroid[e].c[1], q.c[2] - M.centroid[e].c[2]};
        double nr = std::sqrt(r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2]);
        if (nr > mx) mx = nr;
      }
      M.radius.push_back(mx);
      const Vec& q = M.node[M.en[3 * e + 2]];
      M.pplane.push_back(q.c[0] * M.normal[e].c[0] + q.c[1] * M.normal[e].c[1] + q.c[2] * M.normal[e].c[2]);
    }
    M.id = zone;
    M.first = hp.N;
    int mi = (int)meshes.size();
    int ebase = 0;
    for (auto& m : meshes) ebase += (int)m.centroid.size();
    for (int e = 0; e < ne; ++e) {
      double h = (double)(float)hfac * M.radius[e];  // hfac is a float parameter (Contact.cpp:10)
      push(zone, M.centroid[e], 0.0, 0.0, h, 1);
      int p = hp.N - 1;
      for (int d = 0; d < 3; ++d) F(wf::C_NORMAL + d, p) = M.normal[e].c[d];
      hp.i[wf::I_ELEM][p] = ebase + e;
      hp.i[wf::I_MESH][p] = mi;
    }
    meshes.push_back(M);
    return mi;
  }

  // ------------------------------------------------------------ prologue
  void prepare(double dt) {
    using namespace wf;
    int N = hp.N;
    if (N == 0) throw CudaError{WF_ERR_STATE, "no particles"};
    if (!meshes.empty() && !contact) throw CudaError{WF_ERR_ARG, "rigid meshes need contact = 1"};
    if ((int)meshes.size() > MAX_MESHES) throw CudaError{WF_ERR_UNSUPPORTED, "too many rigid meshes"};
    if (solid_part_count < 0) solid_part_count = N;
    for (int p = 0; p < N; ++p) {
      if (hp.i[I_KIND][p] == 0 && p >= solid_part_count)
        throw CudaError{WF_ERR_UNSUPPORTED, "solid particles must precede rigid-mesh particles"};
    }
    CK(cudaSetDevice(device));
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    // CellInitiate (Neighbour.cpp:10-139): bbox of all particles, hmax, pad, cell counts.
    for (int d = 0; d < 3; ++d) { BLPF[d] = F(C_X + d, 0); TRPR[d] = F(C_X + d, 0); }
    hmax = F(C_H, 0);
    double hmin = F(C_H, 0);
    for (int p = 0; p < N; ++p) {
      for (int d = 0; d < 3; ++d) {
        if (F(C_X + d, p) > TRPR[d]) TRPR[d] = F(C_X + d, p);
        if (F(C_X + d, p) < BLPF[d]) BLPF[d] = F(C_X + d, p);
      }
      if (F(C_H, p) > hmax) hmax = F(C_H, p);
      if (F(C_H, p) < hmin) hmin = F(C_H, p);
    }
    for (int d = 0; d < 3; ++d) {
      if (DomMax[d] > TRPR[d]) TRPR[d] = DomMax[d];
      if (DomMin[d] < BLPF[d]) BLPF[d] = DomMin[d];
    }
    for (int d = 0; d < 3; ++d) { TRPR[d] += hmax / 2; BLPF[d] -= hmax / 2; }
    double cs[3];
    long long ncells = 1;
    for (int d = 0; d < 3; ++d) {
      double t = (TRPR[d] - BLPF[d]) / (Cellfac * hmax);
      CellNo[d] = (double(std::ceil(t) - t) < (hmax / 10.0)) ? int(std::ceil(t)) : int(std::floor(t));
      if (CellNo[d] <= 0) throw CudaError{WF_ERR_ARG, "CellInitiate: domain extent smaller than one cell"};
      cs[d] = (TRPR[d] - BLPF[d]) / CellNo[d];
      ncells *= CellNo[d];
    }
    if (ncells > (1LL << 29)) throw CudaError{WF_ERR_UNSUPPORTED, "cell grid too large"};
    // Morton rank of each cell (linear index (i * ny + j) * nz + k).
    std::vector<std::pair<uint64_t, int>> mc((size_t)ncells);
    for (int a = 0; a < CellNo[0]; ++a)
      for (int b = 0; b < CellNo[1]; ++b)
        for (int c = 0; c < CellNo[2]; ++c) {
          int lin = (a * CellNo[1] + b) * CellNo[2] + c;
          mc[lin] = {spread3(a) | (spread3(b) << 1) | (spread3(c) << 2), lin};
        }
    std::sort(mc.begin(), mc.end());
    std::vector<int> rank((size_t)ncells);
    for (long long r = 0; r < ncells; ++r) rank[mc[r].second] = (int)r;

    // Device allocations.
    size_t n = N;
    d_f = dalloc<double>((size_t)NF64 * n);
    d_i = dalloc<int>((size_t)NI32 * n);
    d_fscratch = dalloc<double>((size_t)NF64_PERSIST * n);
    P.g = dalloc<float>((size_t)NF32 * n);
    CK(cudaMemsetAsync(P.g, 0, sizeof(float) * NF32 * n, stream));
    P.rc = reinterpret_cast<float4*>(P.g);
    P.rn = reinterpret_cast<float4*>(P.g + (size_t)4 * RC_N * n);
    P.rates = P.g + (size_t)4 * (RC_N + RN_N) * n;
    d_iscratch = dalloc<int>((size_t)NI32_PERSIST * n);
    CK(cudaMemsetAsync(d_f, 0, sizeof(double) * NF64 * n, stream));
    CK(cudaMemsetAsync(d_i, 0, sizeof(int) * NI32 * n, stream));
    for (int c = 0; c < NF64_PERSIST; ++c)
      CK(cudaMemcpyAsync(d_f + (size_t)c * n, hp.f[c].data(), sizeof(double) * n, cudaMemcpyHostToDevice, stream));
    for (int c = 0; c < NI32_PERSIST; ++c)
      CK(cudaMemcpyAsync(d_i + (size_t)c * n, hp.i[c].data(), sizeof(int) * n, cudaMemcpyHostToDevice, stream));
    P.f = d_f; P.i = d_i;
    P.st = dalloc<StepState>(1);
    DomainTables* tab = dalloc<DomainTables>(1);
    P.tab = tab;
    int* crank = dalloc<int>(ncells);
    CK(cudaMemcpyAsync(crank, rank.data(), sizeof(int) * ncells, cudaMemcpyHostToDevice, stream));
    P.cell_rank = crank;
    {
      std::vector<int> lin(ncells);
      for (size_t c = 0; c < (size_t)ncells; ++c) lin[rank[c]] = (int)c;
      int* clin = dalloc<int>(ncells);
      CK(cudaMemcpyAsync(clin, lin.data(), sizeof(int) * ncells, cudaMemcpyHostToDevice, stream));
      CK(cudaStreamSynchronize(stream));  // the host vector dies at the end of this scope
      P.cell_lin = clin;
    }
    // grid cells, then as many shadow buckets for particles with a non-finite position
    P.cell_start = dalloc<int>(2 * ncells + 1);
    P.cell_count = dalloc<int>(2 * ncells);
    P.perm = dalloc<int>(n);
    P.inv = dalloc<int>(n);
    P.xs = dalloc<float>(4 * n);
    P.row_len = dalloc<int>(n);
    P.row_split = dalloc<int>(n);
    P.nbr = dalloc<int>((size_t)MAX_NB * n);
    P.gk = dalloc<double>((size_t)MAX_NB * n);
    size_t nsb = (n + STAGE_B - 1) / STAGE_B;
    if (stage) {
      CK((cudaError_t)configure_staging(stage_cap));
      P.halo = dalloc<int>(nsb * stage_cap);
      P.halo_len = dalloc<int>(nsb);
      P.nslot = dalloc<unsigned short>((size_t)MAX_NB * n);
      CK(cudaMemsetAsync(P.halo_len, 0, sizeof(int) * nsb, stream));
      stage_ready = true;
    }
    CK(cudaMemsetAsync(P.row_len, 0, sizeof(int) * n, stream));
    CK(cudaMemsetAsync(P.row_split, 0, sizeof(int) * n, stream));
    P.cp_len = dalloc<int>(n);
    CK(cudaMemsetAsync(P.cp_len, 0, sizeof(int) * n, stream));
    P.cp = contact ? dalloc<int>((size_t)MAX_CP * n) : dalloc<int>(1);
    std::vector<int> inv0(n);
    std::iota(inv0.begin(), inv0.end(), 0);
    CK(cudaMemcpyAsync(P.inv, inv0.data(), sizeof(int) * n, cudaMemcpyHostToDevice, stream));
    // Tables.
    DomainTables ht;
    memset(&ht, 0, sizeof(ht));
    ht.nmat = (int)mats.size();
    for (size_t m = 0; m < mats.size(); ++m) ht.mat[m] = mats[m].dev;
    ht.nbc = (int)bcs.size();
    for (size_t b = 0; b < bcs.size(); ++b) {
      BCDev& B = ht.bc[b];
      B.zone = bcs[b].zone; B.value_type = bcs[b].vt; B.amp_id = bcs[b].amp; B.amp_factor = bcs[b].fac;
      for (int d = 0; d < 3; ++d) { B.value[d] = bcs[b].value[d]; B.value_ang[d] = bcs[b].ang[d]; }
    }
    {
      std::vector<int> order(bcs.size());
      std::iota(order.begin(), order.end(), 0);
      std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return bcs[a].zone < bcs[b].zone; });
      int nz = 0;
      for (size_t r = 0; r < order.size(); ++r) {
        ht.bc_order[r] = order[r];
        if (r == 0 || bcs[order[r]].zone != bcs[order[r - 1]].zone) {
          ht.bc_zone[nz] = bcs[order[r]].zone;
          ht.bc_first[nz] = (int)r;
          ++nz;
        }
      }
      ht.bc_first[nz] = (int)order.size();
      ht.bc_nzone = nz;
    }
    ht.namp = (int)amps.size();
    int off = 0;
    for (size_t a = 0; a < amps.size(); ++a) {
      ht.amp[a].id = amps[a].id; ht.amp[a].n = (int)amps[a].t.size(); ht.amp[a].offset = off;
      for (size_t k = 0; k < amps[a].t.size(); ++k) { ht.amp_t[off + k] = amps[a].t[k]; ht.amp_v[off + k] = amps[a].v[k]; }
      off += (int)amps[a].t.size();
    }
    CK(cudaMemcpyAsync(tab, &ht, sizeof(ht), cudaMemcpyHostToDevice, stream));
    // BC particle list (original indices).
    std::vector<int> bl;
    bool any_surface_bc = false;
    for (auto& b : bcs) if (b.zone == 1) any_surface_bc = true;
    const int* zb = ht.bc_zone;
    const int* ze = ht.bc_zone + ht.bc_nzone;
    for (int p = 0; p < N; ++p) {
      bool hit = any_surface_bc && hp.i[I_KIND][p] == 0;
      if (std::binary_search(zb, ze, hp.i[I_ID][p])) hit = true;
      if (hit) bl.push_back(p);
    }
    int* dbl = dalloc<int>(bl.size());
    if (!bl.empty()) CK(cudaMemcpyAsync(dbl, bl.data(), sizeof(int) * bl.size(), cudaMemcpyHostToDevice, stream));
    P.bc_list = dbl;
    // Rigid meshes.
    int nn = 0, ne = 0;
    for (auto& m : meshes) { nn += (int)m.node.size(); ne += (int)m.centroid.size(); }
    P.nnodes = nn; P.nelem = ne;
    std::vector<double> hnode(3 * (size_t)std::max(nn, 1), 0.0), hnorm(3 * (size_t)std::max(ne, 1), 0.0),
        hpp(std::max(ne, 1), 0.0);
    std::vector<int> hen(3 * (size_t)std::max(ne, 1), 0), hem(std::max(ne, 1), 0), hnm(std::max(nn, 1), 0),
        hep(std::max(ne, 1), 0);
    int nb0 = 0, eb0 = 0;
    for (size_t mi = 0; mi < meshes.size(); ++mi) {
      auto& m = meshes[mi];
      for (size_t k = 0; k < m.node.size(); ++k) {
        for (int d = 0; d < 3; ++d) hnode[d * nn + nb0 + k] = m.node[k].c[d];
        hnm[nb0 + k] = (int)mi;
      }
      for (size_t e = 0; e < m.centroid.size(); ++e) {
        for (int k = 0; k < 3; ++k) hen[3 * (eb0 + e) + k] = nb0 + m.en[3 * e + k];
        for (int d = 0; d < 3; ++d) hnorm[d * ne + eb0 + e] = m.normal[e].c[d];
        hpp[eb0 + e] = m.pplane[e];
        hem[eb0 + e] = (int)mi;
        hep[eb0 + e] = m.first + (int)e;
      }
      nb0 += (int)m.node.size();
      eb0 += (int)m.centroid.size();
    }
    P.node = dalloc<double>(hnode.size()); P.node_v = dalloc<double>(hnode.size());
    int* den = dalloc<int>(hen.size()); P.elem_node = den;
    P.elem_normal = dalloc<double>(hnorm.size()); P.elem_pplane = dalloc<double>(hpp.size());
    int* dem = dalloc<int>(hem.size()); P.elem_mesh = dem;
    P.elem_particle = dalloc<int>(hep.size());
    int* dnm = dalloc<int>(hnm.size()); P.node_mesh = dnm;
    CK(cudaMemcpyAsync(P.node, hnode.data(), sizeof(double) * hnode.size(), cudaMemcpyHostToDevice, stream));
    CK(cudaMemsetAsync(P.node_v, 0, sizeof(double) * hnode.size(), stream));
    CK(cudaMemcpyAsync(den, hen.data(), sizeof(int) * hen.size(), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(P.elem_normal, hnorm.data(), sizeof(double) * hnorm.size(), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(P.elem_pplane, hpp.data(), sizeof(double) * hpp.size(), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(dem, hem.data(), sizeof(int) * hem.size(), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(P.elem_particle, hep.data(), sizeof(int) * hep.size(), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(dnm, hnm.data(), sizeof(int) * hnm.size(), cudaMemcpyHostToDevice, stream));
    // Constants.
    K.N = N; K.Nsolid = solid_part_count; K.nbc_particles = (int)bl.size();
    K.Cellfac = Cellfac; K.hmax = hmax; K.dt = dt;
    for (int d = 0; d < 3; ++d) { K.BLPF[d] = BLPF[d]; K.CellSize[d] = cs[d]; K.CellNo[d] = CellNo[d]; }
    // origin of the mixed form's position records: the cell grid's centre
    for (int d = 0; d < 3; ++d) K.rec_origin[d] = BLPF[d] + 0.5 * CellNo[d] * cs[d];
    {
      // Largest pair radius plus a margin over the FP32 rounding of the
      // prefilter coordinates x - BLPF (the grid's extent at most; clamped
      // particles only sit in the outermost cells, whose boxes are unbounded)
      // and of the cell bounds formed in FP32.
      double ext = 0.0;
      for (int d = 0; d < 3; ++d) {
        K.CellSizef[d] = (float)cs[d];
        ext = std::max(ext, CellNo[d] * cs[d]);
      }
      double r = Cellfac * hmax * (1.0 + 1e-5) + 16.0 * 1.1920929e-7 * ext;
      K.cell_skip_r2 = (float)(r * r * (1.0 + 1e-5));
      K.half_cellfac_f = (float)K.Cellfac * 0.5f;
    }
    K.ncells = (int)ncells;
    double ext = 0;
    for (int d = 0; d < 3; ++d) ext = std::max(ext, TRPR[d] - BLPF[d]);
    double R = Cellfac * hmin;
    double eps = 4.0 * std::sqrt(3.0) * std::ldexp(1.0, -23) * (2.0 * ext) / R + 20.0 * std::ldexp(1.0, -24);
    K.pre_eps = (float)(eps < 0.05 ? std::max(eps, 1e-5) : 2.0);
    K.freeze_nb = freeze_nb;
    K.nan_check = nan_check;
    K.nspec = (int)spec_first.size();
    if (K.nspec > 0 && (contact || grad_corr))
      throw CudaError{WF_ERR_UNSUPPORTED, "batched specimens: contact and gradKernelCorr are not supported"};
    // Verlet-skin reuse of the search: on without contact (the contact search
    // bins rigid-mesh particles that move with their planes); the superset
    // radius must stay within two cells and each cell coordinate within 21
    // bits.
    {
      double rmax = Cellfac * hmax, skin = nb_skin * rmax;
      bool fits = true;
      for (int d = 0; d < 3; ++d) fits = fits && CellNo[d] < (1 << 21) && rmax + skin <= 2.0 * cs[d];
      K.skin_on = (nb_skin > 0 && !contact && fits) ? 1 : 0;
      K.skin = K.skin_on ? skin : 0.0;
      double ext2 = 0.0;
      for (int d = 0; d < 3; ++d) ext2 = std::max(ext2, CellNo[d] * cs[d]);
      double r2 = (rmax + skin) * (1.0 + 1e-5) + 16.0 * 1.1920929e-7 * ext2;
      K.sup_skip_r2 = (float)(r2 * r2 * (1.0 + 1e-5));
      // two points within the radius of each other then fall in adjacent cells
      // (ListGenerate's floor((x - BLPF) / CellSize) differs by at most one)
      K.cells_cover = 1;
      for (int d = 0; d < 3; ++d)
        if (!(cs[d] >= rmax * (1.0 + 1e-9))) K.cells_cover = 0;
    }
    K.ts_nb_inc = ts_nb_inc; K.pl_heating = pl_heating; K.thermal_solver = thermal_solver; K.contact = contact;
    K.contact_mesh_auto_update = contact_mesh_auto_update; K.contact_alg = contact_alg;
    K.pl_work_heat_frac = pl_work_heat_frac; K.friction_sta = friction_sta; K.friction_dyn = friction_dyn;
    K.PFAC = PFAC; K.DFAC = DFAC;
    double tm = 0;
    for (int p = 0; p < N; ++p) tm += F(C_MASS, p);
    K.totmass_mean = tm / N;
    K.id_free_surf = -999999;
    K.leapfrog = integrator;
    set_uniform(hp.f[C_ALPHA].data(), hp.f[C_BETA].data(), hp.f[C_MASS].data(), hp.f[C_H].data(),
                hp.f[C_CS].data(), hp.i[I_KIND].data(), hp.i[I_SPEC].data(), N);
    K.gradcorr = grad_corr;
    if (auto_ts_cont && contact && integrator == 0)
      throw CudaError{WF_ERR_UNSUPPORTED, "auto_ts_cont with contact: the kick-drift solver reads Domain::min_force_ts, "
                                          "which nothing on its contact path sets"};
    K.auto_ts = auto_ts; K.auto_ts_acc = auto_ts_acc; K.CFL = CFL; K.sqrt_h_a = sqrt_h_a;
    K.ti = 0;
    for (int p = 0; p < N; ++p)
      if (hp.i[I_KIND][p] == 0 && F(C_TI, p) > 0.0) K.ti = 1;
    K.nmeshes = (int)meshes.size();
    for (size_t m = 0; m < meshes.size(); ++m) K.contact_surf_id[m] = meshes[m].id;
    K.pblock = pblock_now();
    K.fuse_rs = fuse_rs;
    K.nblocks = (N + K.pblock - 1) / K.pblock;
    P.partials = dalloc<double>((size_t)NSLOTS * ((N + 63) / 64));  // room for the smallest block size
    P.scan_tmp = dalloc<long long>((2 * ncells + 4095) / 4096 + 1);
    // Step state.
    StepState st;
    memset(&st, 0, sizeof(st));
    st.deltat = dt; st.prev_deltat = dt; st.deltatint = dt;  // SolverKickDrift.cpp:30
    st.isfirst = 1; st.m_minT = 1000.;
    for (size_t m = 0; m < meshes.size(); ++m)
      for (int d = 0; d < 3; ++d) { st.mesh_v[m][d] = meshes[m].mv.c[d]; st.mesh_w[m][d] = meshes[m].mw.c[d]; }
    CK(cudaMemcpyAsync(P.st, &st, sizeof(st), cudaMemcpyHostToDevice, stream));
    if (K.skin_on) {
      P.sup = dalloc<int>((size_t)SUP_W * n);
      P.sup_len = dalloc<int>(n);
      P.xref = dalloc<double>((size_t)3 * n);
      P.cellc = dalloc<long long>(n);
    }
    if (K.nspec > 0) {  // one rebuild schedule per specimen, as a run of it alone starts
      std::vector<SpecState> sp(K.nspec);
      for (SpecState& q : sp) { memset(&q, 0, sizeof(q)); q.nb_cleared = 1; }
      P.sp = dalloc<SpecState>(K.nspec);
      CK(cudaMemcpyAsync(P.sp, sp.data(), sizeof(SpecState) * K.nspec, cudaMemcpyHostToDevice, stream));
      P.save_len = dalloc<int>(n);
      P.save_nbr = dalloc<int>((size_t)MAX_NB * n);
    }
    regions = {{d_f, sizeof(double) * NF64 * n}, {d_i, sizeof(int) * NI32 * n}, {P.g, sizeof(float) * NF32 * n},
               {P.st, sizeof(StepState)}, {P.inv, sizeof(int) * n}, {P.row_len, sizeof(int) * n},
               {P.row_split, sizeof(int) * n}, {P.nbr, sizeof(int) * MAX_NB * n}, {P.cp_len, sizeof(int) * n},
               {P.cp, contact ? sizeof(int) * MAX_CP * n : sizeof(int)}, {P.node, sizeof(double) * hnode.size()},
               {P.node_v, sizeof(double) * hnode.size()}, {P.elem_normal, sizeof(double) * hnorm.size()},
               {P.elem_pplane, sizeof(double) * hpp.size()}, {P.elem_particle, sizeof(int) * hep.size()}};
    if (stage_ready)
      regions.insert(regions.end(), {{P.halo, sizeof(int) * nsb * stage_cap}, {P.halo_len, sizeof(int) * nsb},
                                     {P.nslot, sizeof(unsigned short) * MAX_NB * n}});
    if (K.nspec > 0) regions.push_back({P.sp, sizeof(SpecState) * K.nspec});
    if (K.skin_on)
      regions.insert(regions.end(), {{P.sup, sizeof(int) * SUP_W * n}, {P.sup_len, sizeof(int) * n},
                                     {P.xref, sizeof(double) * 3 * n}});
    launch_prologue(P, K, stream);
    // SolverKickDrift.cpp:72-96: with contact, a search + CalculateSurface(1)
    // before the loop; the first step searches again (ClearNbData).
    if (contact) {
      launch_force_search(P, stream);
      launch_neighbour_search(P, kconst(), d_fscratch, d_iscratch, stream);
      K.id_free_surf = 1;
    }
    StepState* stp = P.st;
    int one = 1, zero = 0;
    CK(cudaMemcpyAsync(&stp->nb_cleared, &one, sizeof(int), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(&stp->do_search, &zero, sizeof(int), cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
    CK(cudaGetLastError());
    prepared = true;
    check_errors();
  }

  void use_device() { if (prepared) CK(cudaSetDevice(device)); }
  wf::StepState read_state() {
    use_device();
    wf::StepState st;
    CK(cudaMemcpyAsync(&st, P.st, sizeof(st), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    return st;
  }
  void check_errors() {
    wf::StepState st = read_state();
    if (st.errors & wf::ERR_NBR_OVERFLOW) throw CudaError{WF_ERR_NBR_OVERFLOW, "a particle has more than 100 neighbours (MAX_NB_PER_PART)"};
    if (st.errors & wf::ERR_CONTACT_OVERFLOW) throw CudaError{WF_ERR_NBR_OVERFLOW, "a particle has more than 64 contact pairs"};
    if (st.errors & wf::ERR_SPEC_LINK)
      throw CudaError{WF_ERR_ARG, "batch: a neighbour pair links two specimens (they must be spatially apart)"};
    if (st.errors & wf::ERR_TIMEOUT) throw CudaError{WF_ERR_TIMEOUT, "a bounded device wait gave up"};
    if (st.errors & wf::ERR_NAN)
      throw CudaError{WF_ERR_NAN, "non-finite state: a particle position at a neighbour search, or the energy sums"};
    if (contact && st.nb_searches > 0 && st.surface_count == 0)
      throw CudaError{WF_ERR_STATE, "No external particles found. Please check particle masses"};
  }

  // The constants of a launch: K plus the current form and gather block size.
  wf::DomainConst kconst() const {
    wf::DomainConst k = K;
    k.mixed = precision == WF_PRECISION_MIXED;
    k.gblock = gblock_now();
    k.glanes = glanes_now();
    k.pblock = pblock_now();
    k.fuse_rs = fuse_rs;
    k.nblocks = (int)((hp.N + k.pblock - 1) / k.pblock);
    k.stage_cap = stage_ready && stage ? stage_cap : 0;
    return k;
  }
  void launch_one_step() {
    wf::DomainConst k = kconst();
    if (k.mixed) wf::launch_step_mixed(P, k, d_fscratch, d_iscratch, stream);
    else wf::launch_step_fp64(P, k, d_fscratch, d_iscratch, stream);
  }
  // Before running mixed steps: rebuild the float shadows from the FP64 state
  // if plain steps or host writes have touched it since.
  void ensure_shadows() {
    if (precision != WF_PRECISION_MIXED) { shadows_valid = false; return; }
    if (shadows_valid) return;
    wf::DomainConst k = K;
    k.mixed = 1;
    wf::launch_refresh_shadows(P, k, 1, stream);
    shadows_valid = true;
  }
  void step(long long n) {
    if (!prepared) throw CudaError{WF_ERR_STATE, "wf_step before wf_prepare_kickdrift"};
    use_device();
    ensure_shadows();
    if (use_graph) {
      if (!graph || graph_precision != precision || graph_block != graph_key()) capture_step_graph();
      for (long long s = 0; s < n; ++s) CK(cudaGraphLaunch(graph, stream));
    } else {
      for (long long s = 0; s < n; ++s) launch_one_step();
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(stream));
    check_errors();
  }
  double step_timed(long long n, long long* launches) {
    use_device();
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    CK(cudaStreamSynchronize(stream));
    if (use_graph && (!graph || graph_precision != precision || graph_block != graph_key())) step(0);
    ensure_shadows();
    long long l0 = wf::g_launches;
    const long long s0 = search_launches ? read_state().nb_searches : 0;
    CK(cudaEventRecord(a, stream));
    if (use_graph) {
      for (long long s = 0; s < n; ++s) CK(cudaGraphLaunch(graph, stream));
    } else {
      for (long long s = 0; s < n; ++s) launch_one_step();
    }
    CK(cudaEventRecord(b, stream));
    CK(cudaEventSynchronize(b));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    // graph replays: every step's launches, plus the search body's on the
    // steps that searched
    *launches = use_graph ? launches_per_step * n + (search_launches ? search_launches * (read_state().nb_searches - s0) : 0)
                          : wf::g_launches - l0;
    check_errors();
    return ms;
  }
  struct ProfRow { std::string name; double ms; long long count; };
  std::vector<ProfRow> profile(long long n) {
    use_device();
    const int cap = 64 * (int)std::max<long long>(n, 1) + 8;
    std::vector<cudaEvent_t> ev(cap);
    std::vector<const char*> names(cap);
    for (auto& e : ev) CK(cudaEventCreate(&e));
    wf::KernelTimer t;
    t.ev = ev.data(); t.names = names.data(); t.cap = cap; t.n = 0;
    ensure_shadows();
    CK(cudaStreamSynchronize(stream));
    wf::g_timer = &t;
    wf::mark(stream, "begin");
    try {
      for (long long s = 0; s < n; ++s) launch_one_step();
    } catch (...) { wf::g_timer = nullptr; throw; }
    wf::g_timer = nullptr;
    CK(cudaStreamSynchronize(stream));
    std::vector<ProfRow> rows;
    for (int k = 1; k < t.n; ++k) {
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, ev[k - 1], ev[k]));
      auto it = std::find_if(rows.begin(), rows.end(), [&](const ProfRow& r) { return r.name == names[k]; });
      if (it == rows.end()) rows.push_back(ProfRow{names[k], ms, 1});
      else { it->ms += ms; it->count += 1; }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    check_errors();
    return rows;
  }
  void save_to(std::vector<void*>& sl) {
    if (sl.empty())
      for (auto& r : regions) {
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, r.bytes);
        if (e != cudaSuccess) {
          for (void* q : sl) cudaFree(q);
          sl.clear();
          throw CudaError{WF_ERR_NOMEM, std::string("checkpoint: ") + cudaGetErrorString(e)};
        }
        sl.push_back(p);
      }
    for (size_t k = 0; k < regions.size(); ++k)
      CK(cudaMemcpyAsync(sl[k], regions[k].p, regions[k].bytes, cudaMemcpyDeviceToDevice, stream));
    CK(cudaStreamSynchronize(stream));
  }
  void restore_from(const std::vector<void*>& sl) {
    for (size_t k = 0; k < regions.size(); ++k)
      CK(cudaMemcpyAsync(regions[k].p, sl[k], regions[k].bytes, cudaMemcpyDeviceToDevice, stream));
    invalidate_gk();  // the per-entry GradKernel is not part of a checkpoint
    CK(cudaStreamSynchronize(stream));
  }
  // The plain form's per-entry GradKernel (P.gk) no longer matches the state.
  void invalidate_gk() { CK(cudaMemsetAsync(&P.st->gk_valid, 0, sizeof(int), stream)); }
  // Flags of the solid particles' uniform fields, which select the mixed
  // gathers' specialisations and record layout: Alpha and Beta the same on
  // every SPH particle (av_uniform: the pair's (a_i + a_j) / 2 = a from K),
  // the masses of every pair equal (m_pair), and the uniform-particle layout
  // (uni).  spec: each particle's batched specimen (all 0 when the domain is
  // not batched); specimens share no pair, so equal masses within each one
  // make every pair's masses equal.
  void set_uniform(const double* a, const double* b, const double* m, const double* h, const double* cs,
                   const int* kind, const int* spec, size_t n) {
    K.av_uniform = 1;
    K.m_pair = 1;
    bool h_uniform = true, cs_uniform = true;
    bool first = true;
    double a0 = 0, b0 = 0, h0 = 0, c0 = 0;
    const size_t nsp = spec_first.empty() ? 1 : spec_first.size();
    std::vector<double> spec_m(nsp, 0.0);  // first mass seen in each specimen
    std::vector<char> seen(nsp, 0);
    for (size_t p = 0; p < n; ++p) {
      if (kind[p] != 0) continue;
      const int q = spec[p];
      if (!seen[q]) { seen[q] = 1; spec_m[q] = m[p]; }
      else if (m[p] != spec_m[q]) K.m_pair = 0;
      if (first) { a0 = a[p]; b0 = b[p]; h0 = h[p]; c0 = cs[p]; first = false; continue; }
      if (a[p] != a0 || b[p] != b0) K.av_uniform = 0;
      if (h[p] != h0) h_uniform = false;
      if (cs[p] != c0) cs_uniform = false;
    }
    K.av_alpha = (float)a0;
    K.av_beta = (float)b0;
    // the staged gather copies the five-group layout
    K.uni = (K.m_pair && h_uniform && cs_uniform && !stage && h0 > 0) ? 1 : 0;
    K.h_f = (float)h0;
    K.cs_f = (float)c0;
    // the FP32 operations of the per-pair kernel factor at hh = h
    float ih = 1.0f / K.h_f, ih2 = ih * ih;
    K.inv_h_f = ih;
    K.gk_c_f = 0.318309886183790671538f * ih2 * ih2 * ih;
  }
  // Alpha, Beta, mass, h or Cs written after the prologue: re-evaluate the
  // flags on the device columns (any order) and recapture the step with the
  // new constants; the mixed records are rebuilt in the layout they select.
  void refresh_uniform() {
    size_t n = hp.N;
    std::vector<double> a(n), b(n), m(n), h(n), cs(n);
    std::vector<int> kind(n), spec(n);
    CK(cudaMemcpyAsync(a.data(), d_f + (size_t)wf::C_ALPHA * n, sizeof(double) * n, cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(b.data(), d_f + (size_t)wf::C_BETA * n, sizeof(double) * n, cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(m.data(), d_f + (size_t)wf::C_MASS * n, sizeof(double) * n, cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(h.data(), d_f + (size_t)wf::C_H * n, sizeof(double) * n, cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(cs.data(), d_f + (size_t)wf::C_CS * n, sizeof(double) * n, cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(kind.data(), d_i + (size_t)wf::I_KIND * n, sizeof(int) * n, cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(spec.data(), d_i + (size_t)wf::I_SPEC * n, sizeof(int) * n, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    set_uniform(a.data(), b.data(), m.data(), h.data(), cs.data(), kind.data(), spec.data(), n);
    shadows_valid = false;
    if (graph) { CK(cudaGraphExecDestroy(graph)); graph = nullptr; }
  }
  void checkpoint_save(int slot) {
    use_device();
    if ((int)slots.size() <= slot) slots.resize(slot + 1);
    save_to(slots[slot]);
  }
  void checkpoint_restore(int slot) {
    use_device();
    if ((int)slots.size() <= slot || slots[slot].empty()) throw CudaError{WF_ERR_STATE, "checkpoint slot is empty"};
    restore_from(slots[slot]);
  }
  void checkpoint_free(int slot) {
    if ((int)slots.size() <= slot) return;
    for (void* p : slots[slot]) cudaFree(p);
    slots[slot].clear();
  }
  // ------------------------------------------------------------ adjoint
  // Device buffers owned by one adjoint call (freed when it returns).
  struct Scratch {
    std::vector<void*> ps;
    ~Scratch() { for (void* p : ps) cudaFree(p); }
    template <class T> T* get(size_t n) {
      void* p = nullptr;
      cudaError_t e = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T));
      if (e != cudaSuccess) throw CudaError{WF_ERR_NOMEM, std::string("adjoint tape: ") + cudaGetErrorString(e)};
      ps.push_back(p);
      return (T*)p;
    }
  };
  // Fixed-size buffers reused across the segments of one adjoint call.
  template <class T> struct Pool {
    Scratch* sc = nullptr;
    size_t n = 0, used = 0;
    std::vector<T*> bufs;
    T* get() {
      if (used == bufs.size()) bufs.push_back(sc->get<T>(n));
      return bufs[used++];
    }
  };
  struct TapeStep {
    double *start = nullptr, *end = nullptr, *tx = nullptr, *mesh = nullptr;
    int* topo = nullptr;
    bool searched = false;
    double time = 0.0;
  };
  // Topology record layout (ints of N): perm, int arena, row_len, row_split,
  // neighbour rows (MAX_NB), contact count, contact rows (MAX_CP).
  size_t topo_ints() const {
    return (size_t)(3 + wf::NI32_PERSIST + wf::MAX_NB + 1 + (contact ? wf::MAX_CP : 0)) * hp.N;
  }

  // Gradient of a reaction-force loss by the reverse-mode adjoint of the plain
  // FP64 step with checkpoint-and-recompute (see include/weldform_gb300.h).
  void adjoint_reaction(long long steps, int every, int mesh, int axis, const double* target, long long ntarget,
                        int kchk, double* loss, double* grad, double* curve, double* fwd_ms, double* adj_ms) {
    using namespace wf;
    if (!prepared) throw CudaError{WF_ERR_STATE, "adjoint before wf_prepare_kickdrift"};
    if (precision != WF_PRECISION_FP64)
      throw CudaError{WF_ERR_UNSUPPORTED, "the adjoint runs on the plain FP64 form (precision 0)"};
    if (K.ti) throw CudaError{WF_ERR_UNSUPPORTED, "adjoint: tensile instability (TI > 0) is not supported"};
    if (K.leapfrog) throw CudaError{WF_ERR_UNSUPPORTED, "the adjoint differentiates the kick-drift step"};
    if (K.nspec > 0) throw CudaError{WF_ERR_UNSUPPORTED, "adjoint: batched specimens are not supported"};
    if (K.gradcorr) throw CudaError{WF_ERR_UNSUPPORTED, "adjoint: kernel-gradient correction is not supported"};
    if (K.auto_ts || K.auto_ts_acc) throw CudaError{WF_ERR_UNSUPPORTED, "adjoint: the time step must be fixed"};
    if (!contact || mesh < 0 || mesh >= (int)meshes.size())
      throw CudaError{WF_ERR_ARG, "the reaction-force loss needs a rigid mesh"};
    if (axis < 0 || axis > 2 || every < 1 || kchk < 1 || steps < 1 || ntarget < 1 || ntarget * every > steps ||
        !target || !loss || !grad)
      throw CudaError{WF_ERR_ARG, "adjoint: bad steps / sampling / target arguments"};
    size_t n = hp.N;
    {
      std::vector<double> ep(n);
      get_f64(C_EP, 1, ep.data());
      for (double e : ep)
        if (e < 0.0) throw CudaError{WF_ERR_UNSUPPORTED, "adjoint: particles with Ep < 0 are not supported"};
      if (thermal_solver) {
        std::vector<int> bc(n);
        get_i32(I_THBC, bc.data());
        for (int b : bc)
          if (b == 1) throw CudaError{WF_ERR_UNSUPPORTED, "adjoint: convection boundary conditions are not supported"};
      }
    }
    use_device();
    if (use_graph && (!graph || graph_precision != precision || graph_block != graph_key())) step(0);
    Scratch sc;
    double* f0 = sc.get<double>((size_t)NF64_PERSIST * n);
    int* i0 = sc.get<int>((size_t)NI32_PERSIST * n);
    CK(cudaMemcpyAsync(f0, d_f, sizeof(double) * NF64_PERSIST * n, cudaMemcpyDeviceToDevice, stream));
    CK(cudaMemcpyAsync(i0, d_i, sizeof(int) * NI32_PERSIST * n, cudaMemcpyDeviceToDevice, stream));
    double* dF = sc.get<double>(steps);
    long long nseg = (steps + kchk - 1) / kchk;
    std::vector<std::vector<void*>> chk((size_t)nseg + 1);
    struct FreeChk {
      std::vector<std::vector<void*>>& c;
      ~FreeChk() { for (auto& v : c) for (void* p : v) cudaFree(p); }
    } free_chk{chk};
    DomainConst k = kconst();
    k.mixed = 0;

    // ---- forward pass: loss curve and a checkpoint every kchk steps
    auto t0 = std::chrono::steady_clock::now();
    for (long long c = 0; c < nseg; ++c) {
      save_to(chk[c]);
      long long s1 = std::min(steps, (c + 1) * kchk);
      for (long long st = c * kchk; st < s1; ++st) {
        if (use_graph) CK(cudaGraphLaunch(graph, stream));
        else launch_one_step();
        launch_record_force(P, mesh, axis, dF, st, stream);
      }
    }
    save_to(chk[nseg]);
    check_errors();
    auto t1 = std::chrono::steady_clock::now();
    std::vector<double> F(steps);
    CK(cudaMemcpyAsync(F.data(), dF, sizeof(double) * steps, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    double L = 0.0;
    std::vector<double> seed(steps, 0.0);
    for (long long s = 0; s < ntarget; ++s) {
      long long st = (s + 1) * every - 1;
      double r = F[st] - target[s];
      L += r * r;
      seed[st] = 2.0 * r / (double)ntarget;
      if (curve) curve[s] = F[st];
    }
    *loss = L / (double)ntarget;

    // ---- reverse sweep, one recomputed segment at a time
    double* Lin = sc.get<double>((size_t)NA_STATE * n);
    double* Lout = sc.get<double>((size_t)NA_STATE * n);
    double* Tb = sc.get<double>((size_t)NA_TMP * n);
    double* geo = sc.get<double>((size_t)4 * MAX_NB * n);  // pair geometry shared by the adjoint kernels
    double* Q = sc.get<double>((size_t)NQ * n);
    double* Q2 = sc.get<double>((size_t)NQ * n);
    int* derr = sc.get<int>(1);
    CK(cudaMemsetAsync(Lin, 0, sizeof(double) * NA_STATE * n, stream));
    CK(cudaMemsetAsync(Q, 0, sizeof(double) * NQ * n, stream));
    CK(cudaMemsetAsync(derr, 0, sizeof(int), stream));
    Pool<double> snaps{&sc, (size_t)NF64_PERSIST * n}, txs{&sc, (size_t)NTX * n},
        meshp{&sc, (size_t)3 * P.nnodes + P.nelem};
    Pool<int> topos{&sc, topo_ints()};
    std::vector<TapeStep> tape((size_t)std::min<long long>(kchk, steps));
    int nn = P.nnodes, ne = P.nelem;
    auto topo_view = [&](int* t, DevPtrs& S) {
      S.perm = t;
      S.i = t + n;
      S.row_len = S.i + (size_t)NI32_PERSIST * n;
      S.row_split = S.row_len + n;
      S.nbr = S.row_split + n;
      S.cp_len = S.nbr + (size_t)MAX_NB * n;
      S.cp = S.cp_len + n;
    };
    for (long long c = nseg - 1; c >= 0; --c) {
      restore_from(chk[c]);
      snaps.used = txs.used = meshp.used = topos.used = 0;
      long long s0 = c * kchk, s1 = std::min(steps, (c + 1) * kchk);
      double* prev_end = nullptr;
      int* cur_topo = nullptr;
      for (long long st = s0; st < s1; ++st) {
        TapeStep& T = tape[st - s0];
        launch_step_head(P, k, d_fscratch, d_iscratch, stream);
        StepState ss = read_state();
        T.searched = ss.do_search != 0;
        T.time = ss.Time;
        if (T.searched || st == s0) {
          T.topo = topos.get();
          DevPtrs V{};
          topo_view(T.topo, V);
          CK(cudaMemcpyAsync(V.perm, P.perm, sizeof(int) * n, cudaMemcpyDeviceToDevice, stream));
          CK(cudaMemcpyAsync(V.i, d_i, sizeof(int) * NI32_PERSIST * n, cudaMemcpyDeviceToDevice, stream));
          CK(cudaMemcpyAsync(V.row_len, P.row_len, sizeof(int) * n, cudaMemcpyDeviceToDevice, stream));
          CK(cudaMemcpyAsync(V.row_split, P.row_split, sizeof(int) * n, cudaMemcpyDeviceToDevice, stream));
          CK(cudaMemcpyAsync(V.nbr, P.nbr, sizeof(int) * MAX_NB * n, cudaMemcpyDeviceToDevice, stream));
          CK(cudaMemcpyAsync(V.cp_len, P.cp_len, sizeof(int) * n, cudaMemcpyDeviceToDevice, stream));
          if (contact) CK(cudaMemcpyAsync(V.cp, P.cp, sizeof(int) * MAX_CP * n, cudaMemcpyDeviceToDevice, stream));
          cur_topo = T.topo;
          T.start = snaps.get();
          CK(cudaMemcpyAsync(T.start, d_f, sizeof(double) * NF64_PERSIST * n, cudaMemcpyDeviceToDevice, stream));
        } else {
          T.topo = cur_topo;
          T.start = prev_end;
        }
        T.mesh = meshp.get();
        if (nn) CK(cudaMemcpyAsync(T.mesh, P.node, sizeof(double) * 3 * nn, cudaMemcpyDeviceToDevice, stream));
        if (ne) CK(cudaMemcpyAsync(T.mesh + 3 * nn, P.elem_pplane, sizeof(double) * ne, cudaMemcpyDeviceToDevice, stream));
        T.tx = txs.get();
        DevPtrs Pt = P;
        Pt.tx = T.tx;
        launch_step_fp64_body(Pt, k, stream);
        T.end = snaps.get();
        CK(cudaMemcpyAsync(T.end, d_f, sizeof(double) * NF64_PERSIST * n, cudaMemcpyDeviceToDevice, stream));
        prev_end = T.end;
      }
      for (long long st = s1 - 1; st >= s0; --st) {
        TapeStep& T = tape[st - s0];
        AdjPtrs A;
        A.S = P;
        A.S.f = T.start;
        A.S.tx = nullptr;
        topo_view(T.topo, A.S);
        A.S.node = T.mesh;
        A.S.elem_pplane = T.mesh + 3 * nn;
        A.fe = T.end;
        A.tx = T.tx;
        A.Lin = Lin;
        A.Lout = Lout;
        A.Tmp = Tb;
        A.gk_start = geo;
        A.dg_start = geo + (size_t)MAX_NB * n;
        A.gk_end = geo + (size_t)2 * MAX_NB * n;
        A.dg_end = geo + (size_t)3 * MAX_NB * n;
        A.Q = Q;
        A.err = derr;
        A.time = T.time;
        for (int d = 0; d < 3; ++d) A.seed[d] = 0.0;
        A.seed_mesh = -1;
        if (seed[st] != 0.0) { A.seed[axis] = seed[st]; A.seed_mesh = mesh; }
        launch_adjoint_step(A, k, stream);
        if (T.searched) {
          launch_unpermute(A.S.perm, Lout, Lin, NA_STATE, (int)n, stream);
          launch_unpermute(A.S.perm, Q, Q2, NQ, (int)n, stream);
          std::swap(Q, Q2);
        } else {
          std::swap(Lin, Lout);
        }
      }
    }
    DevPtrs P0 = P;
    P0.f = f0;
    P0.i = i0;
    double* dgrad = sc.get<double>(ADJ_NPARAM);
    double* parts = sc.get<double>((size_t)ADJ_NPARAM * ((n + ADJ_BLOCK - 1) / ADJ_BLOCK));
    launch_adjoint_finish(P0, K, Lin, Q, parts, dgrad, stream);
    CK(cudaMemcpyAsync(grad, dgrad, sizeof(double) * ADJ_NPARAM, cudaMemcpyDeviceToHost, stream));
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    CK(cudaGetLastError());
    auto t2 = std::chrono::steady_clock::now();
    restore_from(chk[nseg]);
    if (herr & ERR_ADJ_CONTACT)
      throw CudaError{WF_ERR_UNSUPPORTED, "adjoint: a particle had more than 8 inside contact pairs in one step"};
    if (fwd_ms) *fwd_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    if (adj_ms) *adj_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
  }
  // Launch shape of the mixed gathers: threads per block (64..512) and lanes
  // per particle of the acceleration gather (1, 2, 4), timed over `steps`
  // steps from a checkpoint for every pair; the fastest pair is kept, the
  // state restored, and the choice cached per size bucket (particle count
  // rounded up to a power of two).
  int autotune(int steps) {
    static std::mutex mu;
    static std::map<int, std::pair<int, int>> cache;  // size bucket -> (block, lanes)
    int bucket = 0;
    while ((1LL << bucket) < hp.N) ++bucket;
    {
      std::lock_guard<std::mutex> lk(mu);
      auto it = cache.find(bucket);
      if (it != cache.end()) { gblock = it->second.first; glanes = it->second.second; return gblock; }
    }
    const int slot = 15;
    checkpoint_save(slot);
    int best = 256, best_lanes = 1;
    double best_ms = 1e300;
    for (int lanes : {1, 2, 4, 8})
      for (int b : {64, 128, 256, 512}) {
        gblock = b;
        glanes = lanes;
        long long l = 0;
        step(1);  // capture + warm
        checkpoint_restore(slot);
        double ms = step_timed(steps, &l);
        checkpoint_restore(slot);
        if (ms < best_ms) { best_ms = ms; best = b; best_lanes = lanes; }
      }
    gblock = best;
    glanes = best_lanes;
    checkpoint_free(slot);
    std::lock_guard<std::mutex> lk(mu);
    cache[bucket] = {best, best_lanes};
    return best;
  }
  void search_now() {
    if (!prepared) throw CudaError{WF_ERR_STATE, "neighbour search before the solver prologue"};
    use_device();
    wf::launch_force_search(P, stream);
    wf::launch_neighbour_search(P, kconst(), d_fscratch, d_iscratch, stream);
    shadows_valid = false;  // the search reorders particles
    invalidate_gk();
    int zero = 0;
    CK(cudaMemcpyAsync(&P.st->do_search, &zero, sizeof(int), cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
    check_errors();
  }

  // ------------------------------------------------------------ transfers
  void get_f64(int c, int ncomp, double* dst) {
    size_t n = hp.N;
    if (!prepared) {
      for (size_t p = 0; p < n; ++p)
        for (int k = 0; k < ncomp; ++k) dst[p * ncomp + k] = hp.f[c + k][p];
      return;
    }
    use_device();
    double* tmp = nullptr;
    CK(cudaMallocAsync((void**)&tmp, sizeof(double) * n * ncomp, stream));
    wf::launch_gather_orig(P, K, d_f + (size_t)c * n, tmp, ncomp, stream);
    CK(cudaMemcpyAsync(dst, tmp, sizeof(double) * n * ncomp, cudaMemcpyDeviceToHost, stream));
    CK(cudaFreeAsync(tmp, stream));
    CK(cudaStreamSynchronize(stream));
  }
  // Symmetric (6 stored columns) or antisymmetric (3) tensor as 3x3 rows,
  // expanded on the device so the copy lands straight in dst.
  void get_f64_tensor(int c, int anti, double* dst) {
    size_t n = hp.N;
    use_device();
    double* tmp = nullptr;
    CK(cudaMallocAsync((void**)&tmp, sizeof(double) * n * 9, stream));
    wf::launch_gather_orig_tensor(P, K, d_f + (size_t)c * n, tmp, anti, stream);
    CK(cudaMemcpyAsync(dst, tmp, sizeof(double) * n * 9, cudaMemcpyDeviceToHost, stream));
    CK(cudaFreeAsync(tmp, stream));
    CK(cudaStreamSynchronize(stream));
  }
  // Enqueues a read of column c (ncomp components, or a tensor expanded to
  // 3x3 rows) into dst and returns: the gather runs on the stream in order
  // with the steps, the copy on copy_stream after it.  dst is complete when
  // wf_synchronize returns.
  void get_f64_async(int c, int ncomp, bool tensor, int anti, double* dst) {
    const size_t n = hp.N;
    const size_t bytes = sizeof(double) * n * (tensor ? 9 : ncomp);
    use_device();
    if (!copy_stream) CK(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking));
    Snapshot& sn = snaps[snap_next];
    snap_next = (snap_next + 1) % snaps.size();
    if (!sn.ready) {
      CK(cudaEventCreateWithFlags(&sn.ready, cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&sn.done, cudaEventDisableTiming));
    }
    if (sn.used) CK(cudaStreamWaitEvent(stream, sn.done, 0));  // its last copy has left the buffer
    if (sn.bytes < bytes) {
      if (sn.buf) {
        CK(cudaStreamSynchronize(copy_stream));
        CK(cudaFree(sn.buf));
      }
      sn.buf = nullptr;
      CK(cudaMalloc((void**)&sn.buf, bytes));
      sn.bytes = bytes;
    }
    if (tensor) wf::launch_gather_orig_tensor(P, K, d_f + (size_t)c * n, sn.buf, anti, stream);
    else wf::launch_gather_orig(P, K, d_f + (size_t)c * n, sn.buf, ncomp, stream);
    CK(cudaEventRecord(sn.ready, stream));
    CK(cudaStreamWaitEvent(copy_stream, sn.ready, 0));
    CK(cudaMemcpyAsync(dst, sn.buf, bytes, cudaMemcpyDeviceToHost, copy_stream));
    CK(cudaEventRecord(sn.done, copy_stream));
    sn.used = true;
  }
  void set_f64(int c, int ncomp, const double* src) {
    size_t n = hp.N;
    if (!prepared) {
      for (size_t p = 0; p < n; ++p)
        for (int k = 0; k < ncomp; ++k) hp.f[c + k][p] = src[p * ncomp + k];
      return;
    }
    use_device();
    double* tmp = nullptr;
    CK(cudaMallocAsync((void**)&tmp, sizeof(double) * n * ncomp, stream));
    CK(cudaMemcpyAsync(tmp, src, sizeof(double) * n * ncomp, cudaMemcpyHostToDevice, stream));
    wf::launch_scatter_orig(P, K, tmp, d_f + (size_t)c * n, ncomp, stream);
    CK(cudaFreeAsync(tmp, stream));
    wf::launch_refresh_derived(P, K, stream);
    shadows_valid = false;
    invalidate_gk();
    if (K.skin_on) CK(cudaMemsetAsync(&P.st->sup_valid, 0, sizeof(int), stream));  // positions or h moved
    CK(cudaStreamSynchronize(stream));
    if (c == wf::C_ALPHA || c == wf::C_BETA || c == wf::C_MASS || c == wf::C_H || c == wf::C_CS) refresh_uniform();
  }
  void get_i32(int c, int* dst) {
    size_t n = hp.N;
    if (!prepared) { for (size_t p = 0; p < n; ++p) dst[p] = hp.i[c][p]; return; }
    use_device();
    int* tmp = nullptr;
    CK(cudaMallocAsync((void**)&tmp, sizeof(int) * n, stream));
    wf::launch_gather_orig_i32(P, K, d_i + (size_t)c * n, tmp, stream);
    CK(cudaMemcpyAsync(dst, tmp, sizeof(int) * n, cudaMemcpyDeviceToHost, stream));
    CK(cudaFreeAsync(tmp, stream));
    CK(cudaStreamSynchronize(stream));
  }
  // Canonical-order rows (ELL on device) as CSR over original indices.
  void get_rows(const int* d_len, const int* d_ell, int width, std::vector<long long>& off, std::vector<int>& idx) {
    use_device();
    size_t n = hp.N;
    std::vector<int> len(n), orig(n), ell;
    CK(cudaMemcpyAsync(len.data(), d_len, sizeof(int) * n, cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(orig.data(), d_i + (size_t)wf::I_ORIG * n, sizeof(int) * n, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    int mx = 0;
    for (int l : len) mx = std::max(mx, l);
    mx = std::min(mx, width);
    ell.resize((size_t)mx * n);
    if (mx) CK(cudaMemcpyAsync(ell.data(), d_ell, sizeof(int) * mx * n, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    std::vector<int> sorted_of(n);
    for (size_t i = 0; i < n; ++i) sorted_of[orig[i]] = (int)i;
    off.assign(n + 1, 0);
    for (size_t o = 0; o < n; ++o) off[o + 1] = off[o] + std::min(len[sorted_of[o]], width);
    idx.assign(off[n], 0);
    for (size_t o = 0; o < n; ++o) {
      int i = sorted_of[o];
      int l = std::min(len[i], width);
      for (int k = 0; k < l; ++k) idx[off[o] + k] = orig[wf::nb_index(ell[(size_t)k * n + i])];

    }
  }
};

// ============================================================================ C ABI
namespace {
template <class F> int guard(F&& f) {
  try {
    return f();
  } catch (const CudaError& e) {
    return set_err(e.code, e.msg);
  } catch (const std::exception& e) {
    return set_err(WF_ERR_ARG, e.what());
  } catch (...) {
    return set_err(WF_ERR_ARG, "unknown error");
  }
}
#define NEED(d) if (!(d)) return set_err(WF_ERR_ARG, "null domain")
}  // namespace

extern "C" {

int wf_version(void) { return 10000; }
const char* wf_last_error(void) { return g_err.c_str(); }

int wf_domain_create(int dimension, wf_domain** out) {
  if (!out) return set_err(WF_ERR_ARG, "null out");
  if (dimension != 3) return set_err(WF_ERR_UNSUPPORTED, "only Dimension = 3 is supported");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return set_err(WF_ERR_CUDA, "no CUDA device available");
  *out = new wf_domain();
  return WF_OK;
}
int wf_domain_destroy(wf_domain* d) { delete d; return WF_OK; }

int wf_set_domain_f64(wf_domain* d, const char* name, double v) {
  NEED(d);
  std::string n(name ? name : "");
  if (d->prepared && n != "contact_force_factor") return set_err(WF_ERR_STATE, "domain fields are fixed after the prologue");
  if (n == "Cellfac") d->Cellfac = v;
  else if (n == "pl_work_heat_frac") d->pl_work_heat_frac = v;
  else if (n == "friction_sta") d->friction_sta = v;
  else if (n == "friction_dyn") d->friction_dyn = v;
  else if (n == "PFAC") d->PFAC = v;
  else if (n == "CFL") d->CFL = v;
  else if (n == "sqrt_h_a") d->sqrt_h_a = v;
  else if (n == "DFAC") d->DFAC = v;
  else if (n == "nb_skin") {
    if (!(v >= 0.0 && v <= 0.5)) return set_err(WF_ERR_ARG, "nb_skin must be in [0, 0.5]");
    d->nb_skin = v;
  }
  else if (n == "contact_force_factor") {}
  else if (n.size() == 8 && n.rfind("DomMax.", 0) == 0 && n[7] >= 'x' && n[7] <= 'z') d->DomMax[n[7] - 'x'] = v;
  else if (n.size() == 8 && n.rfind("DomMin.", 0) == 0 && n[7] >= 'x' && n[7] <= 'z') d->DomMin[n[7] - 'x'] = v;
  else return set_err(WF_ERR_ARG, "unknown domain f64 field " + n);
  return WF_OK;
}
int wf_set_domain_i32(wf_domain* d, const char* name, int v) {
  NEED(d);
  std::string n(name ? name : "");
  if (n == "precision") {
    if (v != WF_PRECISION_FP64 && v != WF_PRECISION_MIXED) return set_err(WF_ERR_ARG, "precision must be 0 or 1");
    d->precision = v;
    return WF_OK;
  }
  if (n == "use_graph") { d->use_graph = v != 0; return WF_OK; }
  if (n == "search_conditional") {  // the step graph's search in a conditional IF node
    d->cond_ok = v != 0;
    if (d->graph) { cudaGraphExecDestroy(d->graph); d->graph = nullptr; }  // recapture at the next step
    return WF_OK;
  }
  if (n == "gather_block") {  // 0: by particle count
    if (v != 0 && v != 64 && v != 128 && v != 256 && v != 512)
      return set_err(WF_ERR_ARG, "gather_block must be 0, 64, 128, 256 or 512");
    d->gblock = v;
    return WF_OK;
  }
  if (n == "gather_lanes") {  // lanes per particle of the mixed acceleration gather
    if (v != 1 && v != 2 && v != 4 && v != 8) return set_err(WF_ERR_ARG, "gather_lanes must be 1, 2, 4 or 8");
    d->glanes = v;
    return WF_OK;
  }
  if (n == "gather_staging") {  // shared-memory staged acceleration gather of the mixed form
    if (d->prepared && v && !d->stage_ready)
      return set_err(WF_ERR_STATE, "gather_staging must be set before the prologue (it allocates the halo lists)");
    d->stage = v != 0;
    if (d->prepared)  // the uniform-particle record layout is off while staging is on
      return guard([&] { d->refresh_uniform(); return WF_OK; });
    return WF_OK;
  }
  if (n == "stage_cap") {
    if (d->prepared) return set_err(WF_ERR_STATE, "stage_cap is fixed after the prologue");
    if (v < 64 || v > wf::STAGE_CAP_MAX) return set_err(WF_ERR_ARG, "stage_cap must be in [64, 1024]");
    d->stage_cap = v;
    return WF_OK;
  }
  if (n == "fuse_rate_stress") {  // the step graph is captured again at the next step
    if (v != 0 && v != 1) return set_err(WF_ERR_ARG, "fuse_rate_stress must be 0 or 1");
    d->fuse_rs = v;
    return WF_OK;
  }
  if (n == "particle_block") {  // 0: by particle count
    if (v != 0 && v != 64 && v != 128 && v != 256) return set_err(WF_ERR_ARG, "particle_block must be 0, 64, 128 or 256");
    d->pblock = v;
    return WF_OK;
  }
  if (n == "device") {
    if (d->prepared) return set_err(WF_ERR_STATE, "the device is fixed after the prologue");
    int nd = 0;
    if (cudaGetDeviceCount(&nd) != cudaSuccess || v < 0 || v >= nd) return set_err(WF_ERR_ARG, "no such CUDA device");
    d->device = v;
    return WF_OK;
  }
  if (n == "cpu_threads" || n == "Nproc" || n == "cpu_mode") return WF_OK;
  if (d->prepared) return set_err(WF_ERR_STATE, "domain fields are fixed after the prologue");
  if (n == "ts_nb_inc") { if (v < 1) return set_err(WF_ERR_ARG, "ts_nb_inc >= 1"); d->ts_nb_inc = v; }
  else if (n == "freeze_neighbours") d->freeze_nb = v != 0;
  else if (n == "nan_check") d->nan_check = v != 0;
  else if (n == "pl_heating") d->pl_heating = v;
  else if (n == "thermal_solver") d->thermal_solver = v;
  else if (n == "contact") d->contact = v;
  else if (n == "contact_mesh_auto_update") d->contact_mesh_auto_update = v;
  else if (n == "contact_alg") { if (v < 0 || v > 2) return set_err(WF_ERR_ARG, "contact_alg"); d->contact_alg = v; }
  else if (n == "integrator") {  // 0 SolveDiffUpdateKickDrift, 1 SolveDiffUpdateLeapFrog
    if (v == 2) return set_err(WF_ERR_UNSUPPORTED, "integrator 2 (SolveDiffUpdateFraser) is not built");
    if (v != 0 && v != 1) return set_err(WF_ERR_ARG, "integrator must be 0 (kick-drift) or 1 (leapfrog)");
    d->integrator = v;
  }
  else if (n == "gradKernelCorr") d->grad_corr = v != 0;
  // Domain::h_update (JSON "smoothlenUpdate"): UpdateSmoothingLength
  // (Domain.cpp:2493-2510) runs after each regular search, but both solvers
  // reach it after StartAcceleration zeroed dDensity (Domain.cpp:1586), so it
  // forms htent = h, which fails htent < hmax = h0: h never changes.  The flag
  // is accepted and the step is unchanged (the oracle restates the call).
  else if (n == "h_update") d->h_update = v != 0;
  else if (n == "auto_ts") d->auto_ts = v != 0;          // CheckMinTSVel + AdaptiveTimeStep
  else if (n == "auto_ts_acc") d->auto_ts_acc = v != 0;  // CheckMinTSAccel
  else if (n == "auto_ts_cont") d->auto_ts_cont = v != 0;
  else if (n == "nonlock_sum") { if (!v) return set_err(WF_ERR_UNSUPPORTED, "only the Nishimura sum is supported"); }
  else if (n == "GradientType") { if (v) return set_err(WF_ERR_UNSUPPORTED, "only GradientType 0 is supported"); }
  else return set_err(WF_ERR_ARG, "unknown domain i32 field " + n);
  return WF_OK;
}
int wf_get_domain_f64(wf_domain* d, const char* name, double* v) {
  NEED(d);
  return guard([&] {
    std::string n(name ? name : "");
    if (!d->prepared) {
      if (n == "Time" || n.find("sum") != std::string::npos || n == "plastic_work" || n == "ext_forces_work" ||
          n == "max_pl_strain" || n == "m_maxT" || n == "m_minT") { *v = 0.0; return WF_OK; }
      if (n == "hmax") { *v = 0.0; return WF_OK; }
      if (n == "deltat") { *v = 0.0; return WF_OK; }
      return set_err(WF_ERR_ARG, "unknown domain f64 read " + n);
    }
    wf::StepState st = d->read_state();
    if (n == "Time") *v = st.Time;
    else if (n == "deltat") *v = st.deltat;
    else if (n == "hmax") *v = d->hmax;
    else if (n == "int_energy_sum") *v = st.int_energy_sum;
    else if (n == "kin_energy_sum") *v = st.kin_energy_sum;
    else if (n == "plastic_work") *v = st.plastic_work;
    else if (n == "contact_force_sum") *v = st.contact_force_sum;
    else if (n == "contact_reaction_sum") *v = st.contact_reaction_sum;
    else if (n == "ext_forces_work") *v = st.ext_forces_work;
    else if (n == "max_pl_strain") *v = st.max_pl;
    else if (n == "m_maxT") *v = st.m_maxT;
    else if (n == "m_minT") *v = st.m_minT;
    else return set_err(WF_ERR_ARG, "unknown domain f64 read " + n);
    return WF_OK;
  });
}
int wf_get_domain_i32(wf_domain* d, const char* name, int64_t* v) {
  NEED(d);
  return guard([&] {
    std::string n(name ? name : "");
    if (n == "particle_count") { *v = d->hp.N; return WF_OK; }
    if (n == "solid_part_count") { *v = d->solid_part_count; return WF_OK; }
    if (n == "gather_block") { *v = d->gblock_now(); return WF_OK; }
    if (n == "gather_lanes") { *v = d->glanes_now(); return WF_OK; }
    if (n == "search_conditional") { *v = d->cond_ok ? 1 : 0; return WF_OK; }
    if (n == "particle_block") { *v = d->pblock_now(); return WF_OK; }
    if (n == "fuse_rate_stress") { *v = d->fuse_rs; return WF_OK; }
    if (n == "gather_staging") { *v = d->stage ? 1 : 0; return WF_OK; }
    if (n == "stage_cap") { *v = d->stage_cap; return WF_OK; }
    if (n.size() == 8 && n.rfind("CellNo.", 0) == 0 && n[7] >= 'x' && n[7] <= 'z') { *v = d->CellNo[n[7] - 'x']; return WF_OK; }
    if (!d->prepared) { *v = 0; return WF_OK; }
    if (n == "uniform_layout") { *v = d->K.uni; return WF_OK; }
    if (n == "skin_reuse") { *v = d->K.skin_on; return WF_OK; }
    wf::StepState st = d->read_state();
    if (n == "steps") *v = st.steps;
    else if (n == "pair_count") *v = st.pair_count / 2;
    else if (n == "contact_pair_count") *v = st.contact_pair_count;
    else if (n == "dynamic_friction_count") *v = (int64_t)st.dyn_friction;
    else if (n == "nan_particles") *v = st.nan_count;
    else if (n == "nb_full_searches") *v = st.nb_full_searches;
    else if (n == "nb_searches") *v = st.nb_searches;
    else if (n == "surface_count") *v = st.surface_count;
    else return set_err(WF_ERR_ARG, "unknown domain i32 read " + n);
    return WF_OK;
  });
}
int wf_batch_specimens(wf_domain* d, const int64_t* first, const int64_t* count, int nspec) {
  NEED(d);
  if (d->prepared) return set_err(WF_ERR_STATE, "specimens are fixed after the prologue");
  if (nspec < 1 || !first || !count) return set_err(WF_ERR_ARG, "batch: nspec >= 1 and both arrays are required");
  const int64_t n = d->hp.N;
  std::vector<int> of(n, -1);
  for (int q = 0; q < nspec; ++q) {
    if (first[q] < 0 || count[q] < 1 || first[q] + count[q] > n) return set_err(WF_ERR_ARG, "batch: range out of bounds");
    for (int64_t i = first[q]; i < first[q] + count[q]; ++i) {
      if (of[i] >= 0) return set_err(WF_ERR_ARG, "batch: specimens overlap");
      of[i] = q;
    }
  }
  for (int v : of)
    if (v < 0) return set_err(WF_ERR_ARG, "batch: every particle must belong to a specimen");
  for (int64_t i = 0; i < n; ++i) d->hp.i[wf::I_SPEC][i] = of[i];
  d->spec_first.assign(first, first + nspec);
  d->spec_count.assign(count, count + nspec);
  return WF_OK;
}
int wf_batch_get_i32(wf_domain* d, int spec, const char* name, int64_t* v) {
  NEED(d);
  return guard([&] {
    std::string n(name ? name : "");
    if (spec < 0 || spec >= (int)d->spec_first.size()) return set_err(WF_ERR_ARG, "batch: no such specimen");
    if (n == "first") { *v = d->spec_first[spec]; return WF_OK; }
    if (n == "particle_count") { *v = d->spec_count[spec]; return WF_OK; }
    wf::SpecState q;
    memset(&q, 0, sizeof(q));
    if (d->prepared) {
      d->use_device();
      CK(cudaMemcpyAsync(&q, d->P.sp + spec, sizeof(q), cudaMemcpyDeviceToHost, d->stream));
      CK(cudaStreamSynchronize(d->stream));
    }
    if (n == "nb_searches") *v = q.searches;
    else if (n == "yielding") *v = q.isyielding;
    else return set_err(WF_ERR_ARG, "batch: unknown field " + n);
    return WF_OK;
  });
}
int wf_kernel_set(wf_domain* d, int kt) {
  NEED(d);
  if (kt != 0) return set_err(WF_ERR_UNSUPPORTED, "only the cubic spline kernel (0) is supported");
  d->Cellfac = 2.0;
  return WF_OK;
}
int wf_add_box_length(wf_domain* d, int tag, const double V[3], double Lx, double Ly, double Lz, double r,
                      double density, double h, int type, int rotation, int random, int fixed) {
  NEED(d);
  if (d->prepared) return set_err(WF_ERR_STATE, "particles are fixed after the prologue");
  if (!(type == 0 || type == 1)) return set_err(WF_ERR_ARG, "AddBoxLength: packing type must be 0 or 1");
  if (!(rotation == 0 || rotation == 90)) return set_err(WF_ERR_ARG, "AddBoxLength: rotation must be 0 or 90");
  if (fixed) return set_err(WF_ERR_UNSUPPORTED, "fixed (non-free) particles are not supported");
  if (!(r > 0) || !(h > 0)) return set_err(WF_ERR_ARG, "r and h must be positive");
  if (!d->meshes.empty()) return set_err(WF_ERR_STATE, "add solid particles before rigid meshes");
  d->add_box(tag, V, Lx, Ly, Lz, r, density, h, type, random != 0);
  return WF_OK;
}
int wf_add_cylinder_length(wf_domain* d, int tag, const double V[3], double Rxy, double Lz, double r, double density,
                           double h, int fixed, int ghost) {
  NEED(d);
  if (d->prepared) return set_err(WF_ERR_STATE, "particles are fixed after the prologue");
  if (ghost) return set_err(WF_ERR_UNSUPPORTED, "ghost rows are not supported");
  if (fixed) return set_err(WF_ERR_UNSUPPORTED, "fixed (non-free) particles are not supported");
  if (!(r > 0) || !(h > 0)) return set_err(WF_ERR_ARG, "r and h must be positive");
  if (!d->meshes.empty()) return set_err(WF_ERR_STATE, "add solid particles before rigid meshes");
  d->add_cylinder(tag, V, Rxy, Lz, r, density, h);
  return WF_OK;
}
int wf_assign_zone(wf_domain* d, const double s[3], const double e[3], int id, int64_t* count) {
  NEED(d);
  if (d->prepared) return set_err(WF_ERR_STATE, "zones are fixed after the prologue");
  int64_t c = 0;
  for (int p = 0; p < d->hp.N; ++p) {
    bool in = true;
    for (int k = 0; k < 3; ++k)
      if (d->hp.f[wf::C_X + k][p] < s[k] || d->hp.f[wf::C_X + k][p] > e[k]) in = false;
    if (in) { d->hp.i[wf::I_ID][p] = id; d->hp.i[wf::I_IDORIG][p] = id; d->hp.i[wf::I_NWS][p] = 1; ++c; }
  }
  if (count) *count = c;
  return WF_OK;
}
int wf_set_particle_f64(wf_domain* d, const char* field, int zone, double value) {
  NEED(d);
  if (d->prepared) return set_err(WF_ERR_STATE, "use wf_set_particle_array_f64 after the prologue");
  std::string f(field ? field : "");
  int nc = 0;
  int c = col_f64(f, &nc);
  if (c < 0 || nc != 1) return set_err(WF_ERR_ARG, "unknown particle f64 field " + f);
  for (int p = 0; p < d->hp.N; ++p)
    if (zone < 0 || d->hp.i[wf::I_ID][p] == zone) d->hp.f[c][p] = value;
  return WF_OK;
}
int wf_set_particle_i32(wf_domain* d, const char* field, int zone, int value) {
  NEED(d);
  if (d->prepared) return set_err(WF_ERR_STATE, "particle fields are fixed after the prologue");
  std::string f(field ? field : "");
  int c = col_i32(f);
  if (c < 0 || c == wf::I_NB) {
    std::string why;
    if (!fixed_i32(f, value, &why)) return set_err(c == wf::I_NB ? WF_ERR_ARG : (why.rfind("unknown", 0) == 0 ? WF_ERR_ARG : WF_ERR_UNSUPPORTED), why);
    return WF_OK;
  }
  if (f == "Fail" && value > 1) return set_err(WF_ERR_UNSUPPORTED, "Undefined failure criteria for solids");
  if (f == "Material_model" && (value < 0 || value > 2)) return set_err(WF_ERR_UNSUPPORTED, "material model");
  if (f == "Thermal_BC" && (value < 0 || value > 1))
    return set_err(WF_ERR_UNSUPPORTED, "Thermal_BC: only TH_BC_NONE (0) and TH_BC_CONVECTION (1)");
  for (int p = 0; p < d->hp.N; ++p)
    if (zone < 0 || d->hp.i[wf::I_ID][p] == zone) {
      d->hp.i[c][p] = value;
      if (c == wf::I_ID) d->hp.i[wf::I_IDORIG][p] = value;
    }
  return WF_OK;
}
int wf_set_particle_array_f64(wf_domain* d, const char* field, const double* src, int64_t n) {
  NEED(d);
  return guard([&] {
    std::string f(field ? field : "");
    int nc = 0;
    int c = col_f64(f, &nc);
    if (c < 0) return set_err(WF_ERR_ARG, "unknown particle array " + f);
    if (n != (int64_t)d->hp.N * nc) return set_err(WF_ERR_ARG, "array size mismatch for " + f);
    if (nc == 6 || (nc == 3 && c == wf::C_RR))
      return set_err(WF_ERR_ARG, "tensor fields are set as 9 values per particle");
    d->set_f64(c, nc, src);
    return WF_OK;
  });
}
int wf_get_particle_array_f64(wf_domain* d, const char* field, double* dst, int64_t n) {
  NEED(d);
  return guard([&] {
    std::string f(field ? field : "");
    int nc = 0;
    int c = col_f64(f, &nc);
    if (c < 0) return set_err(WF_ERR_ARG, "unknown particle array " + f);
    size_t N = d->hp.N;
    if (nc == 6 || c == wf::C_RR) {
      if (n != (int64_t)N * 9) return set_err(WF_ERR_ARG, "array size mismatch for " + f);
      if (d->prepared) {
        d->get_f64_tensor(c, nc == 3, dst);
        return WF_OK;
      }
      std::vector<double> t(N * nc);
      d->get_f64(c, nc, t.data());
      for (size_t p = 0; p < N; ++p) {
        double* o = dst + 9 * p;
        const double* s = t.data() + nc * p;
        if (nc == 6) {
          o[0] = s[0]; o[4] = s[1]; o[8] = s[2]; o[1] = o[3] = s[3]; o[2] = o[6] = s[4]; o[5] = o[7] = s[5];
        } else {
          o[0] = o[4] = o[8] = 0.0; o[1] = s[0]; o[3] = -s[0]; o[2] = s[1]; o[6] = -s[1]; o[5] = s[2]; o[7] = -s[2];
        }
      }
      return WF_OK;
    }
    if (n != (int64_t)N * nc) return set_err(WF_ERR_ARG, "array size mismatch for " + f);
    d->get_f64(c, nc, dst);
    return WF_OK;
  });
}
int wf_get_particle_array_f64_async(wf_domain* d, const char* field, double* dst, int64_t n) {
  NEED(d);
  return guard([&] {
    std::string f(field ? field : "");
    int nc = 0;
    int c = col_f64(f, &nc);
    if (c < 0) return set_err(WF_ERR_ARG, "unknown particle array " + f);
    if (!dst) return set_err(WF_ERR_ARG, "null destination");
    const size_t N = d->hp.N;
    const bool tensor = nc == 6 || c == wf::C_RR;
    if (n != (int64_t)N * (tensor ? 9 : nc)) return set_err(WF_ERR_ARG, "array size mismatch for " + f);
    if (!d->prepared) return wf_get_particle_array_f64(d, field, dst, n);  // host arrays: read at once
    d->get_f64_async(c, nc, tensor, nc == 3, dst);
    return WF_OK;
  });
}
int wf_get_particle_array_i32(wf_domain* d, const char* field, int32_t* dst, int64_t n) {
  NEED(d);
  return guard([&] {
    std::string f(field ? field : "");
    if (n != d->hp.N) return set_err(WF_ERR_ARG, "array size mismatch");
    if (f == "IsFree") { for (int p = 0; p < d->hp.N; ++p) dst[p] = 1; return WF_OK; }
    int c = col_i32(f);
    if (c < 0) return set_err(WF_ERR_ARG, "unknown particle i32 array " + f);
    d->get_i32(c, dst);
    return WF_OK;
  });
}
int wf_set_particle_array_i32(wf_domain* d, const char* field, const int32_t* src, int64_t n) {
  NEED(d);
  if (d->prepared) return set_err(WF_ERR_STATE, "integer particle fields are fixed after the prologue");
  std::string f(field ? field : "");
  if (n != d->hp.N) return set_err(WF_ERR_ARG, "array size mismatch");
  int c = f == "not_write_surf_ID" ? wf::I_NWS : col_i32(f);
  if (c < 0 || c == wf::I_NB) return set_err(WF_ERR_ARG, "unknown settable particle i32 array " + f);
  for (int p = 0; p < d->hp.N; ++p) {
    int v = src[p];
    if (f == "Fail" && v > 1) return set_err(WF_ERR_UNSUPPORTED, "Undefined failure criteria for solids");
    if (f == "Material_model" && (v < 0 || v > 2)) return set_err(WF_ERR_UNSUPPORTED, "material model");
    if (f == "Thermal_BC" && (v < 0 || v > 1))
      return set_err(WF_ERR_UNSUPPORTED, "Thermal_BC: only TH_BC_NONE (0) and TH_BC_CONVECTION (1)");
  }
  for (int p = 0; p < d->hp.N; ++p) {
    d->hp.i[c][p] = c == wf::I_NWS ? (src[p] ? 1 : 0) : src[p];
    if (c == wf::I_ID) d->hp.i[wf::I_IDORIG][p] = src[p];
  }
  return WF_OK;
}
int wf_add_material(wf_domain* d, int model, const double* q, int np, int* mat_id) {
  NEED(d);
  if (d->prepared) return set_err(WF_ERR_STATE, "materials are fixed after the prologue");
  if ((int)d->mats.size() >= wf::MAX_MATERIALS) return set_err(WF_ERR_UNSUPPORTED, "too many materials");
  HostMaterial M;
  M.model = model;
  memset(&M.dev, 0, sizeof(M.dev));
  M.dev.model = model;
  if (model == WF_BILINEAR) {
    if (np < 2) return set_err(WF_ERR_ARG, "bilinear needs {E, nu}");
    M.dev.E = q[0];
  } else if (model == WF_HOLLOMON) {
    if (np < 5) return set_err(WF_ERR_ARG, "hollomon needs {E, nu, sy0, K, m}");
    M.dev.E = q[0]; M.dev.sy0 = q[2]; M.dev.K = q[3]; M.dev.m = q[4];
    M.dev.eps0 = q[2] / q[0];                    // Material.cpp:48-57
    M.dev.eps1 = std::pow(q[2] / q[3], 1. / q[4]);
    if (M.dev.eps0 > M.dev.eps1) return set_err(WF_ERR_ARG, "Hollomon material bad definition");
  } else if (model == WF_JOHNSON_COOK) {
    if (np < 10) return set_err(WF_ERR_ARG, "johnson-cook needs {E, nu, A, B, n, C, eps_0, m, T_m, T_t}");
    M.dev.E = q[0]; M.dev.A = q[2]; M.dev.B = q[3]; M.dev.n = q[4]; M.dev.C = q[5]; M.dev.eps_0 = q[6];
    M.dev.jm = q[7]; M.dev.T_m = q[8]; M.dev.T_t = q[9];
  } else {
    return set_err(WF_ERR_UNSUPPORTED, "unknown material model");
  }
  M.p.assign(q, q + np);
  d->mats.push_back(M);
  *mat_id = (int)d->mats.size() - 1;
  return WF_OK;
}
int wf_add_amplitude(wf_domain* d, int id, const double* t, const double* v, int n) {
  NEED(d);
  if (d->prepared) return set_err(WF_ERR_STATE, "amplitudes are fixed after the prologue");
  if (n < 2) return set_err(WF_ERR_ARG, "amplitude needs at least two points");
  int tot = n;
  for (auto& a : d->amps) tot += (int)a.t.size();
  if ((int)d->amps.size() >= wf::MAX_AMPS || tot > wf::MAX_AMP_POINTS) return set_err(WF_ERR_UNSUPPORTED, "amplitude table full");
  d->amps.push_back(HostAmp{id, std::vector<double>(t, t + n), std::vector<double>(v, v + n)});
  return WF_OK;
}
int wf_add_velocity_bc(wf_domain* d, int zone, const double value[3], const double value_ang[3], int value_type,
                       int amp_id, double amp_factor) {
  NEED(d);
  if (d->prepared) return set_err(WF_ERR_STATE, "boundary conditions are fixed after the prologue");
  if ((int)d->bcs.size() >= wf::MAX_BCS) return set_err(WF_ERR_UNSUPPORTED, "too many boundary conditions");
  if (value_type != 0 && value_type != 1) return set_err(WF_ERR_ARG, "value_type must be 0 or 1");
  HostBC b;
  b.zone = zone; b.vt = value_type; b.amp = amp_id; b.fac = amp_factor;
  for (int k = 0; k < 3; ++k) { b.value[k] = value[k]; b.ang[k] = value_ang ? value_ang[k] : 0.0; }
  d->bcs.push_back(b);
  return WF_OK;
}
int wf_add_rigid_plane(wf_domain* d, int axis, int posit, const double p1[3], const double p2[3], int dens,
                       double hfac, int zone_id, int* mesh_id) {
  NEED(d);
  if (d->prepared) return set_err(WF_ERR_STATE, "meshes are fixed after the prologue");
  if (dens <= 0 || axis < 0 || axis > 2) return set_err(WF_ERR_ARG, "bad plane arguments");
  if (zone_id == 1) return set_err(WF_ERR_ARG, "zone id 1 marks the free surface (CalculateSurface(1))");
  if ((int)d->meshes.size() >= wf::MAX_MESHES) return set_err(WF_ERR_UNSUPPORTED, "too many rigid meshes");
  if (d->solid_part_count < 0) d->solid_part_count = d->hp.N;
  int m = d->add_plane(axis, posit != 0, p1, p2, dens, hfac, zone_id);
  if (mesh_id) *mesh_id = m;
  return WF_OK;
}
int wf_set_mesh_velocity(wf_domain* d, int mesh, const double v[3], const double w[3]) {
  NEED(d);
  if (mesh < 0 || mesh >= (int)d->meshes.size()) return set_err(WF_ERR_ARG, "mesh index");
  if (d->prepared) return set_err(WF_ERR_STATE, "set the mesh velocity through a velocity BC after the prologue");
  d->meshes[mesh].mv = vec(v[0], v[1], v[2]);
  if (w) d->meshes[mesh].mw = vec(w[0], w[1], w[2]);
  return WF_OK;
}
int wf_get_contact_force(wf_domain* d, int mesh, double out[3]) {
  NEED(d);
  return guard([&] {
    if (mesh < 0 || mesh >= (int)d->meshes.size()) return set_err(WF_ERR_ARG, "mesh index");
    if (!d->prepared) { out[0] = out[1] = out[2] = 0.0; return WF_OK; }
    wf::StepState st = d->read_state();
    for (int k = 0; k < 3; ++k) out[k] = st.contact_force[mesh][k];
    return WF_OK;
  });
}
int wf_prepare_kickdrift(wf_domain* d, double dt) {
  NEED(d);
  if (d->prepared) return set_err(WF_ERR_STATE, "the prologue already ran");
  if (!(dt > 0)) return set_err(WF_ERR_ARG, "dt must be positive");
  return guard([&] { d->prepare(dt); return WF_OK; });
}
int wf_step(wf_domain* d, int64_t n) {
  NEED(d);
  if (n < 0) return set_err(WF_ERR_ARG, "negative step count");
  return guard([&] { d->step(n); return WF_OK; });
}
int wf_solve_kickdrift(wf_domain* d, double tf, double dt, double dtOut, int64_t maxidx) {
  NEED(d);
  return guard([&] {
    if (!d->prepared) d->prepare(dt);
    // Same loop control as SolverKickDrift.cpp:117,333-346 with Time advanced
    // on the host in the same order as on the device.
    wf::StepState st = d->read_state();
    double Time = st.Time, tout = st.Time;
    int64_t idx_out = 1;
    if (!(d->K.auto_ts || d->K.auto_ts_acc)) {  // fixed dt: the whole loop is known up front
      int64_t pending = 0;
      while (Time <= tf && idx_out <= maxidx) {
        ++pending;
        Time += st.deltat;
        if (Time >= tout) { idx_out++; tout += dtOut; }
      }
      d->step(pending);
      return WF_OK;
    }
    // Adaptive dt never exceeds deltatint, so n = floor((limit - Time) / deltatint)
    // further steps cannot carry Time past the next loop or output boundary:
    // run them as one replay, then read Time back; single steps near a boundary.
    while (Time <= tf && idx_out <= maxidx) {
      double lim = std::min(tf, tout);
      int64_t n = Time < lim ? (int64_t)std::floor((lim - Time) / st.deltatint) : 0;
      if (n > 1) {
        d->step(n - 1);
        st = d->read_state();
        Time = st.Time;
        continue;
      }
      d->step(1);
      st = d->read_state();
      Time = st.Time;
      if (Time >= tout) { idx_out++; tout += dtOut; }
    }
    return WF_OK;
  });
}
int wf_solve_leapfrog(wf_domain* d, double tf, double dt, double dtOut, int64_t maxidx) {
  NEED(d);
  if (d->prepared && d->integrator != 1) return set_err(WF_ERR_STATE, "the domain was prepared for kick-drift");
  d->integrator = 1;
  return wf_solve_kickdrift(d, tf, dt, dtOut, maxidx);
}
int wf_neighbour_search(wf_domain* d) {
  NEED(d);
  return guard([&] { d->search_now(); return WF_OK; });
}
static int rows_out(wf_domain* d, bool contact_rows, int64_t* off, int32_t* idx, int64_t cap) {
  return guard([&] {
    if (!d->prepared) return set_err(WF_ERR_STATE, "no neighbour list yet");
    std::vector<long long> o;
    std::vector<int> ix;
    if (contact_rows) d->get_rows(d->P.cp_len, d->P.cp, d->contact ? wf::MAX_CP : 0, o, ix);
    else d->get_rows(d->P.row_len, d->P.nbr, wf::MAX_NB, o, ix);
    for (size_t k = 0; k < o.size(); ++k) off[k] = o[k];
    if (idx) {
      if (cap < (int64_t)ix.size()) return set_err(WF_ERR_ARG, "idx capacity");
      for (size_t k = 0; k < ix.size(); ++k) idx[k] = ix[k];
    }
    return WF_OK;
  });
}
int wf_get_neighbours(wf_domain* d, int64_t* off, int32_t* idx, int64_t cap) { NEED(d); return rows_out(d, false, off, idx, cap); }
int wf_get_contact_pairs(wf_domain* d, int64_t* off, int32_t* idx, int64_t cap) { NEED(d); return rows_out(d, true, off, idx, cap); }
int wf_step_timed(wf_domain* d, int64_t n, double* ms, int64_t* launches) {
  NEED(d);
  return guard([&] {
    if (!d->prepared) return set_err(WF_ERR_STATE, "wf_step_timed before wf_prepare_kickdrift");
    long long l = 0;
    *ms = d->step_timed(n, &l);
    if (launches) *launches = l;
    return WF_OK;
  });
}
int wf_profile_steps(wf_domain* d, int64_t n, char* names, int name_len, double* total_ms, int64_t* launches,
                     int cap, int* nk) {
  NEED(d);
  return guard([&] {
    if (!d->prepared) return set_err(WF_ERR_STATE, "wf_profile_steps before wf_prepare_kickdrift");
    auto rows = d->profile(n);
    int k = 0;
    for (auto& r : rows) {
      if (k >= cap) break;
      if (names && name_len > 0) {
        strncpy(names + (size_t)k * name_len, r.name.c_str(), name_len - 1);
        names[(size_t)k * name_len + name_len - 1] = 0;
      }
      total_ms[k] = r.ms;
      launches[k] = r.count;
      ++k;
    }
    *nk = k;
    return WF_OK;
  });
}
int wf_checkpoint_save(wf_domain* d, int slot) {
  NEED(d);
  if (slot < 0 || slot > 15) return set_err(WF_ERR_ARG, "checkpoint slot must be 0..15");
  return guard([&] {
    if (!d->prepared) return set_err(WF_ERR_STATE, "checkpoint before the prologue");
    d->checkpoint_save(slot);
    return WF_OK;
  });
}
int wf_checkpoint_restore(wf_domain* d, int slot) {
  NEED(d);
  if (slot < 0 || slot > 15) return set_err(WF_ERR_ARG, "checkpoint slot must be 0..15");
  return guard([&] {
    if (!d->prepared) return set_err(WF_ERR_STATE, "checkpoint before the prologue");
    d->checkpoint_restore(slot);
    return WF_OK;
  });
}
int wf_checkpoint_free(wf_domain* d, int slot) {
  NEED(d);
  if (slot < 0 || slot > 15) return set_err(WF_ERR_ARG, "checkpoint slot must be 0..15");
  d->checkpoint_free(slot);
  return WF_OK;
}
int wf_autotune(wf_domain* d, int steps, int* block) {
  NEED(d);
  if (steps < 1) return set_err(WF_ERR_ARG, "steps >= 1");
  return guard([&] {
    if (!d->prepared) return set_err(WF_ERR_STATE, "autotune before the prologue");
    int b = d->autotune(steps);
    if (block) *block = b;
    return WF_OK;
  });
}
int wf_adjoint_reaction_loss(wf_domain* d, int64_t steps, int every, int mesh, int axis, const double* target,
                             int64_t ntarget, int checkpoint_every, double* loss, double* grad, double* curve,
                             double* fwd_ms, double* adj_ms) {
  NEED(d);
  return guard([&] {
    d->adjoint_reaction(steps, every, mesh, axis, target, ntarget, checkpoint_every, loss, grad, curve, fwd_ms,
                        adj_ms);
    return WF_OK;
  });
}
int wf_synchronize(wf_domain* d) {
  NEED(d);
  return guard([&] {
    if (!d->prepared) return WF_OK;
    d->use_device();
    CK(cudaStreamSynchronize(d->stream));
    if (d->copy_stream) CK(cudaStreamSynchronize(d->copy_stream));
    d->check_errors();
    return WF_OK;
  });
}

}  // extern "C"
