// Device-side data layout of the GB300 kick-drift SPH step (host + device).
//
// Particle state lives in one structure-of-arrays arena in HBM, one column of
// N values per scalar component, in cell-sorted order.  The host keeps the map
// between this order and the reference's particle order ("original index").
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace wf {

// ---- double columns -------------------------------------------------------
// Symmetric tensors are stored as 6 components in the order xx yy zz xy xz yz;
// the reference stores full 3x3 matrices whose off-diagonal pairs agree to the
// last bit except for rounding-order asymmetries of the Jaumann update.
enum F64Col : int {
  C_X = 0,                 // position (3)
  C_V = 3,                 // velocity (3)
  C_RHO = 6,               // Density
  C_A = 7,                 // acceleration (3)
  C_DISP = 10,             // Displacement (3)
  C_MASS = 13, C_RHO0, C_H, C_CS, C_P0, C_G, C_P,
  C_SIG = 20,              // Sigma (6)
  C_TAU = 26,              // ShearStress (6)
  C_EPS = 32,              // Strain (6)
  C_EPL = 38,              // Strain_pl (6)
  C_EPLI = 44,             // Strain_pl_incr (6)
  C_SR = 50,               // StrainRate (6)
  C_PLS = 56, C_DPLS, C_SY, C_EP, C_ESR, C_T, C_DTDT, C_KT, C_CPT, C_THEXP, C_QPL, C_QSRC, C_ALPHA, C_BETA, C_PSEN,
  C_NORMAL = 71,           // normal (3)
  C_CF = 74,               // contforce (3)
  C_DCONT = 77,
  C_DKIN = 78, C_DINT = 79, C_DRHO = 80,
  C_RR = 81,               // RotationRate, antisymmetric part (xy xz yz)
  C_SRHO = 84,             // Sigma / Density^2 (6), for the acceleration pair term
  C_MRHO = 90,             // Mass / Density
  C_PR2 = 91,              // Pressure / Density^2
  C_TI = 92, C_TIN, C_TIDIST,  // tensile instability: TI, TIn, TIInitDist (Particle.h:146-149)
  C_GCM = 95,              // kernel-gradient correction matrix gradCorrM (9, row-major)
  C_TINF = 104,            // convection: T_inf, h_conv and the last q_conv (Particle.h:187)
  C_HCONV = 105,
  C_QCONV = 106,
  NF64_PERSIST = 107,
  // scratch columns (not permuted): next-step buffers and the
  // tensile-instability stress TIR (6), recomputed at every step start
  C_XN = 107, C_VN = 110, C_RHON = 113, C_MRHON = 114, C_TIR = 115,
  C_PR2N = 121,            // next-step Pressure / Density^2 (plain form; read by the fused rate gather)
  C_TN = 122,              // next-step temperature (plain form)
  NF64 = 123
};
enum I32Col : int {
  I_ID = 0, I_IDORIG, I_NWS, I_MAT, I_MODEL, I_FAIL, I_MATERIAL, I_NB, I_KIND, I_ELEM, I_MESH, I_ORIG,
  I_THBC = 12,             // Thermal_BC (Particle.h:69): 1 = convection (TH_BC_CONVECTION)
  I_SPEC = 13,             // specimen of a batched domain (0 otherwise)
  NI32_PERSIST = 14,
  I_CELL = 14,             // scratch: cell key (Morton rank) of the particle at its pre-search position
  I_CLASS = 15,            // scratch: pair-rule class word in sorted order
  NI32 = 16
};

// ---- float4 field groups of the mixed form -----------------------------------
// The FP32 data a neighbour's gather reads is packed four fields to a float4,
// one float4 column per group (group q of particle i at rc[q * N + i]).  In
// cell-sorted order the k-th neighbours of a warp's 32 consecutive particles
// have nearly consecutive indices, so each 16-byte load coalesces into a few
// lines — better than one column per field (more load instructions) and
// better than one record per particle (one line per lane).  Positions,
// velocities and temperature are float-float pairs (hi = fl(v),
// lo = fl(v - hi)); positions are stored relative to a fixed origin O (the
// cell grid's centre), which leaves every difference unchanged.  The six low
// halves of x and v share one group as bf16 values (lo_pack in
// wf_step_common.cuh), so a gather reads three groups per neighbour for x and
// v instead of four.  |lo| is at most half an FP32 ulp of hi and keeps 8
// significant bits, so the difference of two pairs, (hi_i - hi_j) +
// (lo_i - lo_j), carries an absolute error of at most about 2^-33 |x - O|
// besides its FP32 rounding: for a domain of half-extent D that is
// 1.2e-10 D / |x_ij| relative (2e-8 for D = 30 mm at a 0.2 mm spacing, below
// the 6e-8 of the FP32 rounding itself), wherever the domain sits.  A
// velocity difference carries about 2^-33 |v| in the same way.
enum RecCur : int {        // current-state groups
  RC_XH = 0,               // x hi (xyz), h
  RC_L = 1,                // x lo, v lo (bf16 pairs), m/rho
  RC_VH = 2,               // v hi (xyz), rho
  RC_S0 = 3,               // Sigma/rho^2 xx yy zz xy
  RC_S1 = 4,               // Sigma/rho^2 xz yz, mass, Cs
  RC_MISC = 5,             // alpha, beta, k_T, T hi
  RC_T2 = 6,               // T lo
  RC_TI0 = 7,              // TIR xx yy zz xy (tensile instability, when any TI > 0)
  RC_TI1 = 8,              // TIR xz yz, TIn, TIInitDist
  RC_N = 9
};
enum RecNext : int {       // next-step groups
  RN_XH = 0,               // x(n+1) hi, h
  RN_L = 1,                // x(n+1) lo, v(n+1) lo (bf16 pairs), m/rho(n+1)
  RN_VH = 2,               // v(n+1) hi, p/rho^2 at rho(n+1) (the rate gather's kinetic term;
                           // the current group carries rho there)
  RN_E = 3,                // p/rho^2 at rho(n+1), k_T, T(n+1) hi, T(n+1) lo
  RN_N = 4
};
constexpr int NF32 = 4 * (RC_N + RN_N) + 9;  // floats per particle: records + 9 rate columns

struct MaterialDev {
  int model;
  double E;
  double K, m, eps0, eps1, sy0;                         // Hollomon
  double A, B, C, n, jm, eps_0, T_m, T_t;               // Johnson-Cook
};
struct BCDev {
  int zone, value_type, amp_id;
  double value[3], value_ang[3];
  double amp_factor;
};
struct AmpDev {
  int id, n, offset;  // points [offset, offset+n) of the amplitude tables
};

constexpr int MAX_MATERIALS = 512;
constexpr int MAX_BCS = 520;
constexpr int MAX_AMPS = 16;
constexpr int MAX_AMP_POINTS = 512;
constexpr int MAX_MESHES = 8;
constexpr int MAX_NB = 100;  // MAX_NB_PER_PART, Source/Domain.h:49

constexpr int MAX_CP = 64;   // contact pairs per particle
constexpr int SUP_W = 128;   // superset entries per particle (skin reuse of the search)

// Shared-memory staging of the mixed form's gathers.  Particles are taken in
// blocks of STAGE_B consecutive (cell-sorted) particles; at every search each
// block's distinct neighbours are listed once, sorted by index (its halo,
// at most stage_cap of them), and every row entry gets its neighbour's slot
// in that list.  A staged gather copies the halo's float4 groups into shared
// memory once per block and reads neighbours from there.
constexpr int STAGE_B = 128;         // particles (threads) per staged block
constexpr int STAGE_HASH = 4096;     // shared-memory hash set of the halo build
constexpr int STAGE_CAP_MAX = 1024;  // largest halo a block can stage

// Neighbour-row entries: the neighbour's index, bit 31 set when its original
// index is larger than the row particle's (the P2 side of the reference's
// (min, max) pair).  Rows are in the reference's canonical order (j > i
// ascending, then j < i ascending by original index).  On a lattice that order
// lists every interior particle's neighbours by relative offset, so the k-th
// neighbours of a warp's consecutive particles sit at one offset from them:
// ordering rows by memory index instead measured 9 % slower in the gathers.
constexpr unsigned NB_UP = 0x80000000u;
__host__ __device__ __forceinline__ int nb_index(int e) { return e & 0x7fffffff; }
__host__ __device__ __forceinline__ bool nb_up(int e) { return e < 0; }

// Tables that are read by a few threads only; kept in device memory.
struct DomainTables {
  MaterialDev mat[MAX_MATERIALS];
  BCDev bc[MAX_BCS];
  AmpDev amp[MAX_AMPS];
  double amp_t[MAX_AMP_POINTS], amp_v[MAX_AMP_POINTS];
  int nmat, nbc, namp;
  // The BCs grouped by zone: bc_zone[0 .. bc_nzone) the distinct zones
  // ascending; zone z's BCs are bc_order[bc_first[z] .. bc_first[z + 1]) in
  // the order they were added (a later one overrides an earlier one).
  int bc_nzone;
  int bc_zone[MAX_BCS], bc_first[MAX_BCS + 1], bc_order[MAX_BCS];
};

// The range of bc_order holding the BCs of zone id (empty when it has none):
// a binary search over the distinct zones, so a BC particle costs log2 of
// the zone count however many BCs there are.
__device__ __forceinline__ void bc_range(const DomainTables* T, int id, int& lo, int& hi) {
  int a = 0, b = T->bc_nzone;
  while (a < b) {
    int m = (a + b) >> 1;
    if (T->bc_zone[m] < id) a = m + 1; else b = m;
  }
  if (a < T->bc_nzone && T->bc_zone[a] == id) { lo = T->bc_first[a]; hi = T->bc_first[a + 1]; }
  else { lo = 0; hi = 0; }
}

// Error bits raised by kernels (read by the host at synchronisation points).
constexpr int ERR_NBR_OVERFLOW = 1;
constexpr int ERR_NAN = 2;
constexpr int ERR_TIMEOUT = 4;
constexpr int ERR_CONTACT_OVERFLOW = 8;
constexpr int ERR_SPEC_LINK = 16;  // a neighbour pair joins two batched specimens

// Reduction slots (per-block partials, deterministic tree order).
enum Slot : int {
  S_DINT = 0, S_DKIN, S_PLW, S_MAXPL, S_MAXT, S_MINT, S_CFSUM, S_CRSUM, S_EXTW,
  S_DTV = 9,    // CheckMinTSVel's smallest candidate time step (block minima)
  S_DTA = 10,   // CheckMinTSAccel's
  S_CFVEC = 11, // 3 per mesh
  NSLOTS = 11 + 3 * MAX_MESHES
};

// Scalars that evolve on the device, so a whole step runs without a host sync.
struct StepState {
  double Time, deltat;
  double prev_deltat;  // the step's time step before AdaptiveTimeStep (first kick; leapfrog kick)
  double deltatint;    // the solver's initial time step (Domain::deltatint)
  double int_energy_sum, kin_energy_sum, plastic_work, contact_force_sum, contact_reaction_sum, ext_forces_work;
  double max_pl;       // max pl_strain at the start of the current step
  double max_pl_next;  // max pl_strain after the current step's stress update
  double m_maxT, m_minT;
  double mesh_v[MAX_MESHES][3];         // TriMesh::m_v set by the velocity BCs
  double mesh_w[MAX_MESHES][3];         // TriMesh::m_w
  double contact_force[MAX_MESHES][3];  // Domain::m_contact_force
  long long steps, nb_searches;
  unsigned long long pair_count, contact_pair_count;
  int isfirst, isyielding, ts_i, nb_cleared;
  int do_search;       // set by the schedule kernel for the current step
  int do_gradcorr;     // recompute the kernel-gradient correction this step
  int gk_valid;        // P.gk holds GradKernel at the current positions and rows (plain form:
                       // the last step's rate pass formed it; host writes, restores and
                       // searches clear it)
  int errors;
  int surface_count;
  unsigned long long dyn_friction;  // contact-pair evaluations that took the dynamic-friction branch
  // Verlet-skin reuse of the neighbour search (DomainConst::skin_on)
  unsigned long long maxdisp2_bits;  // largest squared displacement since the superset was built (as bits)
  int search_full;     // this step's search re-sorts and rebuilds the superset (else: filter only)
  int sup_valid;       // a superset exists and every row fitted in SUP_W
  long long nb_full_searches;
  int nan_count;       // particles with a non-finite position at the last search
};

// Rebuild schedule of one specimen of a batched domain: the state a run of
// that specimen alone keeps (SolverKickDrift.cpp:153-186, 315-324).
struct SpecState {
  int yielded_next;    // a particle of the specimen has pl_strain > MIN_PS_FOR_NBSEARCH (after this step)
  int yielded;         // ... at the start of the current step
  int isyielding, ts_i, nb_cleared;
  int do_search;       // the specimen searches this step
  long long searches;
};

// Per-domain constants (set once at the solver prologue; small, by value).
struct DomainConst {
  int N, Nsolid, nbc_particles;
  double Cellfac, hmax, dt;
  double BLPF[3], CellSize[3];
  int CellNo[3];
  double rec_origin[3];  // the mixed form's position records hold x - rec_origin (the cell grid's centre)
  int ncells;
  float pre_eps;       // relative margin of the FP32 neighbour prefilter
  float cell_skip_r2;  // (Cellfac * hmax + FP32 rounding margin)^2: cells farther hold no neighbour
  float CellSizef[3];  // FP32 copy of the cell size
  float half_cellfac_f;  // 0.5 * Cellfac in FP32 (prefilter radius factor)
  int ts_nb_inc, pl_heating, thermal_solver, contact, contact_mesh_auto_update, contact_alg;
  double pl_work_heat_frac, friction_sta, friction_dyn, PFAC, DFAC;
  double totmass_mean;
  int id_free_surf;
  int nmeshes;
  int contact_surf_id[MAX_MESHES];
  int pblock;          // threads per block of the per-particle kernels (64, 128 or 256)
  int nblocks;         // blocks of the per-particle kernels at pblock (partials stride)
  int fuse_rs;         // mixed form, one lane per particle: rate gather and stress update in one kernel
  int mixed;           // 1 when the step runs the mixed FP32/FP64 kernels
  int gblock;          // thread-block size of the mixed form's gather kernels
  int glanes;          // lanes per particle of the mixed acceleration gather (1, 2, 4 or 8)
  int ti;              // 1 when some particle has TI > 0 (tensile-instability term on)
  int leapfrog;        // 1: SolveDiffUpdateLeapFrog's update (velocities at half steps)
  int gradcorr;        // 1: kernel-gradient correction (Domain::gradKernelCorr)
  int auto_ts, auto_ts_acc;  // adaptive time step: velocity / acceleration criteria
  double CFL, sqrt_h_a;      // their coefficients (Domain::CFL, Domain::sqrt_h_a)
  int av_uniform;      // 1 when every solid particle has the same Alpha and Beta
  float av_alpha, av_beta;  // those values (the mixed acceleration gather skips their loads)
  // 1 when the two particles of every pair have the same mass: the mass is
  // uniform, or uniform within each batched specimen (no pair links two
  // specimens, ERR_SPEC_LINK).  The gathers then take m_j = m_i.
  int m_pair;
  // Uniform-particle layout of the mixed records: every solid particle has the
  // same h and Cs, the pairs' masses agree (m_pair), and the staged gather is
  // off.  The current records then carry Sigma/rho^2 xz in RC_XH.w and yz in
  // RC_VH.w (instead of h and rho), so the acceleration gather reads four
  // groups per neighbour instead of five, rho_j = m_i / (m/rho)_j, and every
  // gather uses the kernel constants of the one h below instead of forming
  // 1/h per pair.
  int uni;
  float h_f, cs_f;     // that h and Cs
  float inv_h_f;       // 1 / h
  float gk_c_f;        // 1 / (pi h^5): the 3D cubic spline's gradient factor GK = gk_c_f * w(q)
  int stage_cap;       // halo capacity of the staged gathers (0: staging off)
  int freeze_nb;       // 1: neighbour and contact topology searched only at the first step
  int nan_check;       // 1: a non-finite position at a search, or non-finite energy sums, raise ERR_NAN
  int nspec;           // batched specimens with their own rebuild schedules (0: one schedule)
  // Verlet-skin reuse of the search: a full search also lists, per particle,
  // every particle within its pair radius plus `skin` (canonical order); a
  // later search whose particles have all moved less than skin / 2 since then
  // filters those lists with the exact pair rules instead of re-sorting.
  int skin_on;
  double skin;         // absolute skin length
  float sup_skip_r2;   // squared largest superset radius plus margin, in FP32 (cell pruning)
  int cells_cover;     // every cell is wider than the largest pair radius (with a 1e-9 margin)
};

// Device pointers, passed by value to every kernel.
struct DevPtrs {
  double* f;         // F64 arena: column c at f + c * N
  int* i;            // I32 arena
  float* g;          // F32 arena of the mixed form: current groups, next groups, 9 rate columns
  float4* rc;        // current-state float4 groups (RC_N columns of N)
  float4* rn;        // next-step float4 groups (RN_N columns of N)
  float* rates;      // StrainRate (6) + RotationRate (3) columns
  StepState* st;
  const DomainTables* tab;
  const int* cell_rank;   // linear cell -> Morton rank
  const int* cell_lin;    // Morton rank -> linear cell
  int* cell_start;        // ncells + 1
  int* cell_count;        // ncells (histogram / cursor)
  int* perm;              // new sorted position -> old sorted position
  int* inv;               // original index -> sorted position
  float* xs;              // FP32 prefilter coordinates (x - BLPF, 3 columns) and h
  int* row_len;           // neighbours per particle
  int* row_split;         // neighbours with larger original index (row prefix)
  int* nbr;               // ELL: entry k of particle i at k * N + i
  double* gk;             // plain form: GradKernel per row entry (same ELL layout) at the
                          // current positions: written by the rate pass at x(n+1) (or by the
                          // acceleration pass when stale), read by the next step's
                          // acceleration and density passes
  int* cp_len;            // contact pairs per particle
  int* cp;                // ELL, width MAX_CP
  const int* bc_list;     // original indices of particles carrying a BC zone id
  // rigid meshes
  double* node;           // 3 * nnodes (SoA: x[nnodes], y, z)
  double* node_v;
  const int* elem_node;   // 3 * nelem
  double* elem_normal;    // 3 * nelem
  double* elem_pplane;    // nelem
  const int* elem_mesh;   // nelem
  int* elem_particle;     // nelem -> sorted particle index
  const int* node_mesh;   // nnodes
  int nnodes, nelem;
  int* halo;              // staged gathers: each STAGE_B block's neighbours, sorted (stage_cap per block)
  int* halo_len;          // per block: halo size, -1 when above stage_cap (that block reads global memory)
  unsigned short* nslot;  // ELL like nbr: the entry's slot in its block's halo
  double* partials;       // NSLOTS * nblocks
  long long* scan_tmp;
  double* tx;             // step tape of the adjoint's recompute (TapeCol columns), null otherwise
  int* sup;               // skin: superset rows (ELL width SUP_W, canonical order, NB_UP flag)
  int* sup_len;
  double* xref;           // skin: positions when the superset was built (3 columns)
  long long* cellc;       // skin: cell coordinates at the current search (21 bits each; -1 if not finite)
  SpecState* sp;          // batched domain: one schedule per specimen
  int* save_len;          // batched domain: rows of the specimens that do not search, kept across
  int* save_nbr;          // the search's reordering (original indices, ELL by old position)
};

// Per-step values the plain form writes for the adjoint when DevPtrs::tx is
// set: the inputs of the contact and density passes and the branch record of
// the radial return, so the reverse pass takes exactly the forward branches.
enum TapeCol : int {
  TX_APRE = 0,             // acceleration entering the contact pass (after the first BC pass) (3)
  TX_VH = 3,               // half-step velocity entering the density pass (3)
  TX_SR = 6,               // StrainRate before the thermal-expansion term (6)
  TX_RR = 12,              // RotationRate (xy xz yz)
  TX_SC = 15,              // radial-return scale min(Sigmay / sig_trial, 1)
  TX_SYN = 16,             // flow stress recomputed in the step (JC / Hollomon; Sigmay otherwise)
  TX_DEP = 17,             // plastic strain increment (0 when elastic)
  NTX = 18
};

}  // namespace wf
