/*
 * weldform_gb300 — C ABI of the GB300 (sm_103a) explicit SPH solid step.
 *
 * This is the drop-in boundary for WeldForm's kick-drift solid path.  The
 * reference has no plugin or FFI layer: its "API" is the public members of
 * SPH::Domain, SPH::Particle, the Material_ classes and TriMesh, compiled into
 * each executable.  Every entry point below names the reference member it
 * replaces (paths relative to the WeldForm source tree).
 *
 * Conventions
 *  - Every call returns an int status (WF_OK == 0).  wf_last_error() gives a
 *    human-readable message for the last failing call on this thread.
 *    No exception ever crosses the ABI (the reference throws `new Fatal`,
 *    External/fatal.h:58-63, or calls abort(), Functions.cpp:64-70).
 *  - Particles are addressed in the reference's insertion order ("original
 *    index"); the library reorders them internally (cell-sorted) and maps
 *    indices back on every host transfer.
 *  - Vectors are passed as double[3]; per-particle arrays as flat host
 *    buffers (n * components, row-major).  The library copies inputs and
 *    never keeps a caller pointer.
 *  - One host thread per domain; one CUDA stream per domain.
 *  - SI units, exactly as the reference (no unit conversion anywhere).
 */
#ifndef WELDFORM_GB300_H
#define WELDFORM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define WF_OK               0
#define WF_ERR_ARG          1  /* invalid argument / unknown field name          */
#define WF_ERR_CUDA         2  /* CUDA runtime error or no device                 */
#define WF_ERR_NAN          3  /* non-finite value detected in the state          */
#define WF_ERR_NBR_OVERFLOW 4  /* a particle exceeds the neighbour cap (100,
                                  MAX_NB_PER_PART, Source/Domain.h:49)           */
#define WF_ERR_TIMEOUT      5  /* a bounded device wait gave up                   */
#define WF_ERR_STATE        6  /* call not valid in the current solver state      */
#define WF_ERR_NOMEM        7  /* device or host allocation failed                */
#define WF_ERR_UNSUPPORTED  8  /* reference feature outside this build's scope   */

/* ---- precision forms ------------------------------------------------------ */
#define WF_PRECISION_FP64   0  /* plain form: FP64 throughout                     */
#define WF_PRECISION_MIXED  1  /* FP32 Kahan pair sums, FP64 integration/return   */

/* ---- material models (Source/Particle.h:34-37) ---------------------------- */
#define WF_BILINEAR      0
#define WF_HOLLOMON      1
#define WF_JOHNSON_COOK  2

/* ---- contact stiffness laws ------------------------------------------------ */
#define WF_CONTACT_WANG    0  /* kij = 2 m / dt^2, Source/Contact_Wang.cpp:187      */
#define WF_CONTACT_PENALTY 1  /* kij = PFAC * cont_stiff, Source/Contact.cpp:423;
                                 cont_stiff per Source/SolverKickDrift.cpp:79-84   */
#define WF_CONTACT_AREA    2  /* kij = PFAC * (m/rho)^(2/3): a pressure-per-length
                                 penalty times the particle contact area
                                 (Source/Contact_Wang.cpp:248 gives the area)     */

typedef struct wf_domain wf_domain;

/* Library version (major*10000 + minor*100 + patch). */
int wf_version(void);
/* Message of the last failing call on this thread ("" if none). */
const char* wf_last_error(void);

/* Domain::Domain (Source/Domain.cpp:78-175).  dimension must be 3. */
int wf_domain_create(int dimension, wf_domain** out);
/* Domain::~Domain (Source/Domain.cpp:177-181).  Frees host and device state. */
int wf_domain_destroy(wf_domain* d);

/* Domain scalar fields (Source/Domain.h:113-537).  Names are the reference
 * member names: "Cellfac", "pl_work_heat_frac", "friction_sta",
 * "friction_dyn", "PFAC", "DFAC", "CFL", "sqrt_h_a", "DomMax.x|y|z",
 * "DomMin.x|y|z", "contact_force_factor", "nb_skin" (Verlet skin of the
 * neighbour-search reuse, a fraction of the largest pair radius, default 0.1,
 * 0 off; no reference counterpart: a full search also lists every particle
 * within the pair radius plus the skin, and a later search whose particles
 * have all moved less than half the skin since filters those lists with the
 * exact pair rules instead of re-sorting — the rows are the same; on without
 * contact and without batched specimens).  Integer fields: "Nproc", "ts_nb_inc",
 * "nonlock_sum", "pl_heating", "thermal_solver", "contact",
 * "contact_mesh_auto_update", "GradientType", "contact_alg" (WF_CONTACT_*),
 * "integrator" (0 kick-drift, 1 leapfrog; before the prologue; 2, the
 *   Fraser order of SolveDiffUpdateFraser, is WF_ERR_UNSUPPORTED),
 * "gradKernelCorr" (kernel-gradient correction, Domain.cpp:1832-1940; plain
 * FP64 form; the correction matrix is recomputed at the first step and, for
 * the leapfrog solver, after every rebuild),
 * "auto_ts", "auto_ts_acc", "auto_ts_cont" (adaptive time step after the
 * contact pass, SolverKickDrift.cpp:216-219 / SolverLeapfrog.cpp:257-260:
 * CheckMinTSVel, CheckMinTSAccel, AdaptiveTimeStep, Domain.cpp:206-319; the
 * step never exceeds the solver's initial dt; auto_ts_cont with contact in
 * the kick-drift solver is WF_ERR_UNSUPPORTED, as it reads a member nothing
 * on that path sets; f64 fields "CFL" (default 0.7) and "sqrt_h_a" (0.0025)
 * are the criteria's coefficients; read the current step with "deltat"),
 * "h_update" (Domain::h_update: UpdateSmoothingLength, Domain.cpp:2493-2510,
 * after each regular rebuild; both solvers reach it with dDensity already
 * zeroed by StartAcceleration, so h does not change: accepted, no effect),
 * "precision" (WF_PRECISION_*), "device" (CUDA device ordinal, before the
 * prologue), "use_graph" (replay each step as one CUDA graph, default 1),
 * "search_conditional" (1: the graph's neighbour search sits in a conditional
 * node, so a step without a search launches none of its kernels; default 0,
 * as ncu cannot profile the kernel nodes of such a graph),
 * "gather_block" (threads per block of the mixed form's gathers: 64, 128,
 * 256 or 512), "gather_lanes" (lanes per particle of the mixed acceleration
 * gather: 1, 2, 4 or 8; the lanes walk one row and combine their Kahan
 * partials by warp shuffles; the density and rate gathers use the same
 * lanes; by default 8 below 20,000 particles, 4 below 40,000, 2 below
 * 64,000, else 1), "gather_staging" (1: the mixed acceleration gather reads each
 * 128-particle block's neighbours from a shared-memory copy of their records,
 * built at every search; set before the prologue, default 0) and
 * "stage_cap" (its halo capacity per block, 64..1024, default 896, before
 * the prologue), "freeze_neighbours" (1: neighbour rows, contact pairs and
 * surface flags come from the first step's search only, for finite-difference
 * checks of the adjoint; no reference counterpart), "nan_check" (1: a
 * particle position that is not finite at a neighbour search, or non-finite
 * energy sums, make the next status-returning call fail with WF_ERR_NAN;
 * default 0 keeps the reference's behaviour of stepping on with NaN; no
 * reference counterpart; before the prologue), "particle_block" (threads
 * per block of the per-particle kernels: 64, 128 or 256; 0, the default,
 * chooses by particle count), "fuse_rate_stress" (mixed form with one lane
 * per particle: 1, the default, runs the rate gather and the stress update as
 * one kernel, 0 as two; the results are bit-identical; no reference
 * counterpart; any time), "cpu_threads" and "cpu_mode" (the CPU
 * restatement's thread count and structure; accepted and unused on the GPU
 * path).  Read back with wf_get_domain_i32: "gather_block", "gather_lanes",
 * "particle_block", "fuse_rate_stress", "gather_staging", "stage_cap",
 * "search_conditional". */
int wf_set_domain_f64(wf_domain* d, const char* name, double value);
int wf_set_domain_i32(wf_domain* d, const char* name, int value);
/* Read-back of scalars: "Time", "deltat", "hmax", "int_energy_sum",
 * "kin_energy_sum", "plastic_work", "contact_force_sum",
 * "contact_reaction_sum", "ext_forces_work", "max_pl_strain", "m_maxT",
 * "m_minT"; integers: "particle_count", "solid_part_count", "steps",
 * "pair_count", "contact_pair_count", "nb_searches", "CellNo.x|y|z",
 * "surface_count", "nb_full_searches" (searches that re-sorted the particles;
 * the rest filtered the skin lists), "dynamic_friction_count" (contact-pair evaluations since
 * the prologue that took the dynamic-friction branch, Contact_Wang.cpp:284-290;
 * no reference counterpart), "nan_particles" (particles whose position was not
 * finite at the last neighbour search: they get empty rows and appear in no
 * row, as CheckRadius decides for them, without being binned into a cell),
 * "uniform_layout" (1 when the mixed records take the four-group
 * uniform-particle layout: h and Cs uniform, and every pair's masses equal —
 * uniform, or uniform within each batched specimen), "skin_reuse" (1 when the
 * Verlet-skin reuse of the search is on). */
int wf_get_domain_f64(wf_domain* d, const char* name, double* value);
int wf_get_domain_i32(wf_domain* d, const char* name, int64_t* value);

/* Domain::Kernel_Set (Source/Domain.cpp:190-194).  Only Qubic_Spline (0). */
int wf_kernel_set(wf_domain* d, int kernel_type);

/* Domain::AddBoxLength (Source/Domain.h:127-128, Source/Domain.cpp:326-599).
 * 3D packings: type 1 cubic, type 0 hexagonal close packing. */
int wf_add_box_length(wf_domain* d, int tag, const double V[3], double Lx, double Ly,
                      double Lz, double r, double density, double h, int type,
                      int rotation, int random, int fixed);
/* Domain::AddCylinderLength (Source/Domain.h:130-131, Source/Domain.cpp:708-860). */
int wf_add_cylinder_length(wf_domain* d, int tag, const double V[3], double Rxy,
                           double Lz, double r, double density, double h, int fixed,
                           int ghost);
/* Domain::AssignZone (Source/Domain.h:495, Source/Domain.cpp:691-706). */
int wf_assign_zone(wf_domain* d, const double start[3], const double end[3], int id,
                   int64_t* count);

/* Per-particle public fields (Source/Particle.h:50-265) for every particle
 * whose ID equals `zone`, or all particles when zone < 0.
 * f64 fields: "G", "Cs", "Sigmay", "Ep", "Alpha", "Beta", "TI", "TIn", "TIInitDist",
 * "k_T", "cp_T", "T", "th_exp", "Density", "RefDensity", "Mass", "h", "P0",
 * "q_source", "T_inf", "h_conv".  i32 fields: "PresEq", "Fail",
 * "Material_model", "mat", "Material", "ID", "IsFree", "print_history",
 * "Thermal_BC" (1 = TH_BC_CONVECTION: with the thermal solver on, every step
 * sets q_conv = rho h_conv (m/rho)^(2/3) (T_inf - T) / m after the temperature
 * update and adds it to dTdt, CalcConvHeat, Thermal.cpp:339-389; the JSON
 * driver's "ConvectionBC" sets these three per zone, WeldForm.cpp:793-807). */
int wf_set_particle_f64(wf_domain* d, const char* field, int zone, double value);
int wf_set_particle_i32(wf_domain* d, const char* field, int zone, int value);
/* Whole-array transfer in original particle order.  Vector fields ("x", "v",
 * "a", "Displacement", "normal", "contforce") take 3 values per particle;
 * tensor fields ("Sigma", "ShearStress", "StrainRate", "RotationRate",
 * "Strain", "Strain_pl", "Strain_pl_incr", "TIR" read-only, "gradCorrM"
 * read-only) 9 (row-major, full 3x3, as the reference stores them); scalars
 * 1 ("Density", "Pressure", "pl_strain", "Sigmay", "T", "dTdt",
 * "eff_strain_rate", "q_plheat", "q_conv", "Mass", "h", "delta_pl_strain",
 * "dDensity", "delta_cont" (contact penetration), "dint_energy_dt",
 * "dkin_energy_dt" (the particles' energy rates), "ps_energy" (accumulated
 * plastic work per volume)) and every per-particle f64 field above.  n is the
 * total number of doubles. */
int wf_set_particle_array_f64(wf_domain* d, const char* field, const double* src,
                              int64_t n);
int wf_get_particle_array_f64(wf_domain* d, const char* field, double* dst, int64_t n);
/* The same read, asynchronous: the field is snapshotted on the device in order
 * with the steps already enqueued and copied to dst on a copy stream while
 * later steps run; dst holds the values once wf_synchronize returns (up to
 * four reads may be in flight; a fifth waits for the oldest).  dst must stay
 * valid until then; pinned host memory lets the copy overlap the steps. */
int wf_get_particle_array_f64_async(wf_domain* d, const char* field, double* dst, int64_t n);
/* Integer arrays: "ID", "Nb", "IsFree", "Thermal_BC". */
int wf_get_particle_array_i32(wf_domain* d, const char* field, int32_t* dst, int64_t n);
/* Per-particle integer fields as whole arrays, before the prologue: "ID",
 * "mat", "Material_model", "Fail", "Material", "not_write_surf_ID", "Thermal_BC"
 * (Particle.h:50-265; the array form of assigning them in a loop). */
int wf_set_particle_array_i32(wf_domain* d, const char* field, const int32_t* src, int64_t n);

/* Materials (Source/Material.h:64-224, Source/Material.cpp:6-72).
 * model WF_BILINEAR: params {E, nu}            (hardening via particle Ep)
 * model WF_HOLLOMON: params {E, nu, sy0, K, m} (Material.cpp:48-57)
 * model WF_JOHNSON_COOK: params {E, nu, A, B, n, C, eps_0, m, T_m, T_t}
 *   (JohnsonCook ctor order, Material.h:124-131).
 * Returns the material index to put in the particle field "mat". */
int wf_add_material(wf_domain* d, int model, const double* params, int nparams,
                    int* mat_id);

/* Amplitude table (SPH::amplitude, Source/Domain.h:69-89). */
int wf_add_amplitude(wf_domain* d, int id, const double* time, const double* value,
                     int n);
/* Velocity boundary condition in the form the JSON driver's UserAcc applies
 * (Source/WeldForm.cpp:51-120): particles with ID == zone get a = 0 and
 * v = value (value_type 0) or amp_factor * amplitude(t) * value (value_type 1);
 * a rigid mesh whose id == zone gets m_v (and m_w = value_ang). The callback
 * runs at the three reference call sites (Source/SolverKickDrift.cpp:208,231,267). */
int wf_add_velocity_bc(wf_domain* d, int zone, const double value[3],
                       const double value_ang[3], int value_type, int amp_id,
                       double amp_factor);

/* Rigid plane contact surface: TriMesh::AxisPlaneMesh (Source/Mesh.cpp:82-203),
 * TriMesh::CalcSpheres (Mesh.cpp:206-220) and Domain::AddTrimeshParticles
 * (Source/Contact.cpp:10-38) in one call.  Returns the mesh index.  zone_id
 * may not be 1: the solver marks free-surface particles with id 1
 * (CalculateSurface(1), SolverKickDrift.cpp:94), and a mesh with that id would
 * pair surface particles with each other (WF_ERR_ARG). */
int wf_add_rigid_plane(wf_domain* d, int axis, int positaxisorent, const double p1[3],
                       const double p2[3], int dens, double hfac, int zone_id,
                       int* mesh_id);
/* TriMesh::SetVel / SetRotAxisVel (Source/Mesh.h:68-69). */
int wf_set_mesh_velocity(wf_domain* d, int mesh, const double v[3], const double w[3]);
/* Domain::m_contact_force[mesh] (Source/Contact_Wang.cpp:312). */
int wf_get_contact_force(wf_domain* d, int mesh, double out[3]);

/* Domain::SolveDiffUpdateKickDrift (Source/Domain.h:199,
 * Source/SolverKickDrift.cpp:23-401) without file output: runs the prologue
 * (if not yet run) and steps while Time <= tf && idx_out <= maxidx. */
int wf_solve_kickdrift(wf_domain* d, double tf, double dt, double dtOut, int64_t maxidx);
/* Domain::SolveDiffUpdateLeapFrog (Source/Domain.h:200,
 * Source/SolverLeapfrog.cpp:24-451): the same prologue and rebuild schedule
 * with the leapfrog update (velocities at half steps: the first step starts
 * from v - a dt/2, then v += a dt; density and drift with v(n+1/2), rates at
 * x(n+1), v(n+1/2)).  Equivalent to wf_set_domain_i32(d, "integrator", 1)
 * before the prologue followed by wf_solve_kickdrift. */
int wf_solve_leapfrog(wf_domain* d, double tf, double dt, double dtOut, int64_t maxidx);
/* The solver prologue only (SolverKickDrift.cpp:23-115, identical for the
 * leapfrog solver) with time step dt. */
int wf_prepare_kickdrift(wf_domain* d, double dt);
/* Advance exactly nsteps kick-drift steps (SolverKickDrift.cpp:117-393). */
int wf_step(wf_domain* d, int64_t nsteps);

/* Neighbour search at the current positions (Neighbour.cpp:141-257 cell
 * assignment + Neighbour.cpp:346-477 search + CalcPairPosList :617-694).
 * Valid after wf_prepare_kickdrift. */
int wf_neighbour_search(wf_domain* d);
/* The current same-material pair list (SMPairs) as CSR in original indices,
 * each row in canonical order: j > i ascending, then j < i ascending (the
 * Anei layout, Neighbour.cpp:672-675).  offsets has particle_count+1 entries;
 * idx holds at most cap entries (call with idx == NULL to get the size in
 * offsets[particle_count]). */
int wf_get_neighbours(wf_domain* d, int64_t* offsets, int32_t* idx, int64_t cap);
/* Contact pairs (ContPairs, Contact.cpp:57-132): row = solid particle,
 * entries = rigid-mesh particles, ascending; same calling convention. */
int wf_get_contact_pairs(wf_domain* d, int64_t* offsets, int32_t* idx, int64_t cap);

/* ---- batched specimens (no counterpart in the reference, which runs one
 * domain per process) ---------------------------------------------------------
 * Partitions the particles, by original index, into nspec specimens
 * [first[s], first[s] + count[s]) that are stepped together in every launch
 * but each keep the rebuild schedule a run of that specimen alone would have
 * (SolverKickDrift.cpp:153-186, 315-324: the first step, the first step with a
 * particle past MIN_PS_FOR_NBSEARCH, then every ts_nb_inc steps while
 * yielding).  A search serves the specimens that ask for one; the others keep
 * their rows (with the Verlet-skin reuse, most searches filter the skin lists
 * of the asking specimens instead of re-sorting the domain).  Specimens must
 * be spatially apart: a neighbour pair that joins two of them fails the step
 * with WF_ERR_ARG.  Each specimen may have its own mass; with equal masses
 * within each one the mixed records keep the uniform-particle layout.  Every
 * particle must belong to exactly one specimen; before the prologue; contact
 * and gradKernelCorr are WF_ERR_UNSUPPORTED, and so is the adjoint on such a
 * domain. */
int wf_batch_specimens(wf_domain* d, const int64_t* first, const int64_t* count, int nspec);
/* Per-specimen read-back: "nb_searches" (searches the specimen asked for),
 * "yielding" (1 once it has yielded), "first", "particle_count". */
int wf_batch_get_i32(wf_domain* d, int spec, const char* name, int64_t* value);

/* Blocks until the domain's streams are idle (steps and asynchronous reads)
 * and reports deferred device status (non-finite state, neighbour overflow,
 * bounded-wait timeout). */
int wf_synchronize(wf_domain* d);

/* ---- device checkpoints ----------------------------------------------------
 * The reference's restart reads positions only (Input.cpp:4-97); these keep
 * the complete solver state (particle arena, neighbour and contact lists,
 * rigid meshes, step scalars) in device memory, in up to 16 slots, so a run
 * can be rewound (recompute-based adjoints, tuning runs, what-if branches).
 * A slot is allocated on its first save and reused afterwards. */
int wf_checkpoint_save(wf_domain* d, int slot);
int wf_checkpoint_restore(wf_domain* d, int slot);
int wf_checkpoint_free(wf_domain* d, int slot);

/* Chooses the launch shape of the mixed form's gather kernels — threads per
 * block (64, 128, 256 or 512) and lanes per particle of the gathers (1, 2,
 * 4 or 8) — by timing `steps` steps with every pair from a
 * checkpoint of the current state, restores that state, keeps the fastest and
 * returns its block size; results are cached per size bucket (particles
 * rounded up to a power of two) for later domains in the process.  The choice
 * is also domain fields "gather_block" and "gather_lanes", settable after the
 * prologue. */
int wf_autotune(wf_domain* d, int steps, int* block);

/* ---- reaction-force adjoint (no counterpart in the reference) ------------
 * Gradient of the loss
 *     L = (1/S) sum_s (F(s) - target[s])^2,
 * F(s) = component `axis` of the contact force on rigid mesh `mesh`
 * (Domain::m_contact_force, Contact_Wang.cpp:312) after step (s+1)*every of a
 * run of `steps` steps from the current state, S = ntarget,
 * with respect to the parameters (grad[WF_NPARAM], in this order):
 *   WF_P_E     Young's modulus, through G = E/(2(1+nu)) and
 *              Cs = sqrt(E/(3(1-2nu)rho0)) of every particle (dt fixed)
 *   WF_P_SY0   initial Sigmay of bilinear / Hollomon particles
 *   WF_P_EP    Ep of every particle (bilinear hardening modulus)
 *   WF_P_A .. WF_P_M   Johnson-Cook A, B, n, C, m of every material, including
 *              their effect on the initial Sigmay = CalcYieldStress(0, 0, T0)
 *              (WeldForm.cpp:905-906)
 *   WF_P_MU    friction_sta = friction_dyn
 *   WF_P_PFAC  contact stiffness factor (contact_alg 1 and 2)
 * The plain FP64 step (precision 0) is differentiated in reverse mode with the
 * neighbour and contact lists of each step frozen.  The forward run stores a
 * device checkpoint every `checkpoint_every` steps; the reverse sweep
 * recomputes one segment at a time, taping its steps, and runs the adjoint
 * kernels backwards over it.  On return the domain holds the state after
 * `steps` steps, as if wf_step had run them.  curve (optional, ntarget values)
 * receives F(s); fwd_ms / adj_ms (optional) the wall time of the forward run
 * and of the reverse sweep.  Errors: WF_ERR_UNSUPPORTED for the mixed form,
 * particles with Ep < 0 or convection boundary conditions. */
#define WF_NPARAM 10
enum { WF_P_E = 0, WF_P_SY0, WF_P_EP, WF_P_A, WF_P_B, WF_P_N, WF_P_C, WF_P_M, WF_P_MU, WF_P_PFAC };
int wf_adjoint_reaction_loss(wf_domain* d, int64_t steps, int every, int mesh, int axis, const double* target,
                             int64_t ntarget, int checkpoint_every, double* loss, double* grad, double* curve,
                             double* fwd_ms, double* adj_ms);

/* ---- measurement helpers (no counterpart in the reference) ---------------
 * wf_step_timed: nsteps steps bracketed by CUDA events recorded on the
 * domain's stream (synchronised before and after); elapsed_ms is the event
 * time, kernel_launches the number of this library's kernels launched.
 * wf_profile_steps: nsteps steps launched one kernel at a time with an event
 * after every kernel; per distinct kernel name (at most cap, name_len bytes
 * each in names) the summed milliseconds and launch count. */
int wf_step_timed(wf_domain* d, int64_t nsteps, double* elapsed_ms, int64_t* kernel_launches);
int wf_profile_steps(wf_domain* d, int64_t nsteps, char* names, int name_len, double* total_ms,
                     int64_t* launches, int cap, int* nkernels);

/* ---- fixed-footprint neighbour search (no counterpart in the reference) ---
 * For callers that cannot allocate device memory (code running inside a
 * memory pool owned by another library, plugin hosts that forbid device
 * allocations, real-time loops where an allocation may stall or fail): the
 * same cell-list search and radius rule as a domain rebuild, over
 * caller-owned device buffers, with its working memory in one file-scope
 * device array of fixed size (about 10 MB per GPU that loads the library,
 * held until exit).
 * x, y, z, h: n device doubles each; the cell grid as CellInitiate computes it
 * (BLPF, CellSize, CellNo; Neighbour.cpp:10-139) and Cellfac.  Outputs:
 * row_len[n] and nbr (device, n * 100 ints, entry k of particle i at
 * k * n + i, rows ordered j > i ascending then j < i ascending).  A row with
 * more than 100 neighbours gets length 101 and holds its 100 smallest keys
 * (the reference writes past its arrays there; a domain rebuild reports
 * WF_ERR_NBR_OVERFLOW instead).  Work is enqueued on `stream` (a cudaStream_t,
 * NULL for the default stream); nothing is allocated or freed.  Limits:
 * n <= WF_STATIC_MAX_PARTICLES and CellNo.x * CellNo.y * CellNo.z <=
 * WF_STATIC_MAX_CELLS, else WF_ERR_ARG.  All calls share the one array: calls
 * that overlap on the GPU race.  The first call on a device resolves the
 * array's address with that device current — make it before any stream
 * capture; the look-up is repeated after the device's context has been
 * re-created (cudaDeviceReset). */
#define WF_STATIC_MAX_PARTICLES 262144
#define WF_STATIC_MAX_CELLS 1048576
int wf_neighbour_list_static(const double* x, const double* y, const double* z, const double* h,
                             int64_t n, const double blpf[3], const double cell_size[3],
                             const int32_t cell_no[3], double cellfac, int32_t* row_len,
                             int32_t* nbr, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* WELDFORM_GB300_H */
