/*
 * parmec_gb300.h -- C ABI of the GB300 (sm_103a) implementation of Parmec's
 * explicit DEM time step.
 *
 * Two surfaces are exported by libparmec_gb300.so:
 *
 *  (1) Compat entry points with the exact names and argument lists of the ISPC
 *      exports that Parmec's host loop calls (parmec.cpp:2386-2517).  Each takes
 *      host structure-of-arrays pointers, copies them to a device mirror, runs
 *      the CUDA kernels and copies the results back, so an unmodified parmec.cpp
 *      can link against this library instead of the ISPC objects.  They are
 *      declared inside namespace ispc for C++ callers, as ISPC's generated
 *      headers do (parmec.cpp:46-55).
 *
 *  (2) A device-resident session API (pg_session_*): the whole scene lives in
 *      HBM, one call advances many steps.  This is what the Python DEM()
 *      command and the benchmarks use.
 *
 * All REAL arguments are double (the reference's -DREAL=8 build, macros.h:60).
 * Every function returns an int status (PG_OK, or a negative PG_ERR_*) where the
 * reference would have called ASSERT/exit.  No function falls back to the CPU:
 * without a CUDA device they return PG_ERR_CUDA.
 */
#ifndef PARMEC_GB300_H
#define PARMEC_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define PG_OK                 0
#define PG_ERR_CUDA         (-1)  /* a CUDA runtime call failed */
#define PG_ERR_CAPACITY     (-2)  /* a per-particle list overflowed; the session re-sizes and re-runs */
#define PG_ERR_ARGUMENT     (-3)  /* invalid argument (size, index, null pointer) */
#define PG_ERR_UNSUPPORTED  (-4)  /* a case the reference asserts on (ellipsoids, USER_FORCE) */
#define PG_ERR_TIMEOUT      (-5)  /* a bounded device wait gave up */

/* ---- constants shared with the reference (constants.h:33-64) ------------- */
#define PG_NIPARAM 7              /* SPRING, DAMPER, FRISTAT, FRIDYN, FRIROL, FRIDRIL, KSKN */
#define PG_SPRING_NONLINEAR_ELASTIC 0
#define PG_SPRING_GENERAL_NONLINEAR 1
#define PG_SPRING_YIELDED   1
#define PG_SPRING_UNLOADING 2
#define PG_SPRDIR_CONSTANT  4
#define PG_SPRDIR_PLANAR    8
#define PG_SPRDIR_FOLLOWER  16
#define PG_SPRDIR_PROJECT   32
#define PG_FLAG_ANALYTICAL  1
#define PG_FLAG_OUTREST     2
#define PG_FLAG_SKIP        4

/* ---- reference-defect switches (pg_scene.compat bits) -------------------- */
/* expmap's v02 = Omega2*Omega3 typo (macros.h:1505); ON reproduces it.        */
#define PG_COMPAT_EXPMAP    1
/* moving obstacle k's contacts read obstacle k+1's point and velocity
 * (input.cpp:1391,1433 vs forces.ispc:265); ON reproduces it.                 */
#define PG_COMPAT_OBSIDX    2
/* triangle_sphere's region s >= 0, t < 0, s+t >= det, a+d <= b+e takes the
 * ac-edge parameter -e/c for s (condet.ispc:371-375, 597-601), so a centre
 * beyond vertex b is matched to vertex a; ON reproduces it, OFF uses the
 * ab-edge parameter -d/a.                                                     */
#define PG_COMPAT_TRIEDGE   4

/*
 * Host description of one scene: the reference's global SoA buffers
 * (parmec.cpp:61-285) as plain pointers.  One pointer per vector component,
 * exactly like the reference (e.g. position[0..2] current, [3..5] reference;
 * rotation is a column-major 3x3, macros.h:945).  Arrays a scene does not use
 * may be NULL when their count is zero.
 */
typedef struct pg_scene {
  /* particles (parmec.cpp:95-114) */
  int parnum;
  double *angular[6];   /* [0..2] referential Omega, [3..5] spatial omega */
  double *linear[3];
  double *rotation[9];
  double *position[6];
  double *inertia[9];
  double *inverse[9];
  double *mass;
  double *invm;
  double *force[3];
  double *torque[3];
  int *flags;
  int *parmat;

  /* spheres (parmec.cpp:86-93); radii[1] < 0 marks a sphere */
  int ellnum;
  double *center[6];
  double *radii[3];
  int *ellcol;
  int *part;

  /* triangles (parmec.cpp:116-121): tri[vertex][coord][index] */
  int trinum;
  double *tri[3][3];
  int *tricol;
  int *triobs;          /* -1 static, -k-2 moving obstacle k, >=0 mesh particle */

  /* moving obstacles */
  int obsnum;
  int *trirng;          /* [2*obsnum] triangle ranges */
  double *obspnt;       /* [3*obsnum] rotation points (updated by obstacles) */
  double *obsang;       /* [3*obsnum] current angular velocities (last obstaclev) */
  double *obslin;       /* [3*obsnum] current linear velocities (last obstaclev) */

  /* surface pairing (sorted by sort_materials, parmec.cpp:1636) */
  int pairnum;
  int *pairs;           /* [2*pairnum] colour pairs */
  int *ikind;           /* [pairnum] GRANULAR_FORCE = 0 */
  double *iparam[PG_NIPARAM];

  /* meshed particles: nodes and faces (parmec.cpp nodes/facnod/factri) */
  int nodnum;
  double *nodes[6];     /* [0..2] current, [3..5] reference */
  int *nodpart;
  int facnum;
  int *facnod[3];
  int *factri;

  /* translational springs, sorted by (part0, part1) (parmec.cpp:151-178) */
  int sprnum;
  int *sprtype;
  int *unspring;
  int *sprpart[2];
  double *sprpnt[2][6];
  double *spring[2];  int *spridx;
  double *dashpot[2]; int *dashidx;
  double *unload[2];  int *unidx;
  double *yield[2];
  double *sprdir[6];
  int *sprflg;
  int *sproffset;
  double *sprfric;
  double *sprkskn;
  double *sprsdsp[3];
  double *stroke0;
  double *stroke[3];
  double *sprfrc[3];
  double *lcurve[2];  int *lcidx;

  /* prescribed motion (input.cpp:2647-2795); values come per step */
  int prsnum;
  int *prspart;
  int *prslin;          /* 1 when the linear motion is prescribed */
  int *prsang;          /* 1 when the angular motion is prescribed */
  int *linkind;         /* 0 velocity, 1 acceleration */
  int *angkind;

  int compat;           /* PG_COMPAT_* bits */

  /* independent scenes sharing one session (batching and serving pools);
   * nscene == 0 means a single scene and the arrays below may be NULL */
  int nscene;
  int *pscene;          /* [parnum] scene of each particle */
  int *tscene;          /* [trinum] scene of each triangle (a scene's triangles are contiguous) */
  int *oscene;          /* [obsnum] scene of each obstacle */
  int *sactive;         /* [nscene] 1 when the scene steps */

  /* restraints (RESTRAIN, input.cpp:2458-2644): particle, then three linear
   * and three angular orthonormal directions (zero rows where fewer are
   * given) along which velocities (at each DEM call) and forces (each step)
   * lose their components (restrain.ispc:30-133) */
  int rstnum;
  int *rstpart;
  double *rstlin[9];
  double *rstang[9];

  /* spring failure rules (UNSPRING, input.cpp:2083-2295; unspring_task,
   * forces.ispc:2058-2127).  Spring lists hold spring ids (creation order),
   * mapped to sorted positions through sprmap.  unent uses the reference's
   * history codes (PG_HIS_STROKE .. PG_HIS_FF), unop its operator codes.
   * nfreq counts failures down and is written back by pg_session_download;
   * unaction is -1 (zero force) or an lcurve index (unload curve). */
  int unsprnum;
  int *tsprings, *tspridx;   /* tested springs, CSR over rules */
  int *msprings, *mspridx;   /* monitored springs: fail when the rule fires */
  int *activate, *actidx;    /* springs switched on when the rule fires */
  double *unlim[2];          /* lower, upper limit */
  int *unent, *unop, *unabs, *nsteps, *nfreq, *unaction;
  int *sprmap;               /* [sprnum] spring id -> sorted position */

  /* torsion springs (TORSION_SPRING, input.cpp:1791-2080), sorted by
   * (part0, part1) (sort_trqspr, parmec.cpp:1968); krpy/drpy are per-axis
   * (roll, pitch, yaw) lookup tables, a one-entry damper table is a critical
   * damping ratio; trqcone holds the TRQCONE_* flags (constants.h:66-68);
   * zdir1/xdir1, the angles and the moments are state written by the step */
  int trqsprnum;
  int *trqsprpart[2];
  double *trqzdir0[3], *trqxdir0[3];
  double *krpy[3][2]; int *krpyidx[3];
  double *drpy[3][2]; int *drpyidx[3];
  int *trqcone;
  double *trqzdir1[3], *trqxdir1[3];
  double *trqrpy[3], *trqrpytot[3], *trqrpyspr[3];

  /* externally prescribed body forces (parmec.h:281-289, applied by
   * prescribe_body_forces, parmec.cpp:2202-2224): one record per particle;
   * each step the particle's force and torque after forces() are exported to
   * pbfin (inner: force xyz, torque xyz; written back by
   * pg_session_download) and pbfout (outer) is added to them */
  int pbfnum;
  int *pbfpart;
  double *pbfout[6];
  double *pbfin[6];
} pg_scene;

/* UNSPRING entity and operator codes (constants.h:43-46, 70) */
#define PG_HIS_STROKE 25
#define PG_HIS_F      26
#define PG_HIS_SF     27
#define PG_HIS_FF     28
#define PG_OP_SUM     0
#define PG_OP_MAX     1
#define PG_OP_MIN     2

/*
 * Per-step host inputs of the time loop.  The reference evaluates these through
 * Python callbacks or TSERIES inside the loop (input.cpp:4199-4503); the host
 * samples them at the same times before the steps run.  Row s belongs to step
 * s of this call.  NULL means "zero for every step".
 */
typedef struct pg_steptab {
  int nsteps;
  const double *curtime;   /* [n]  time at the start of each step */
  const double *gravity;   /* [n][3] at curtime */
  const double *damping;   /* [n][6] at curtime */
  const double *prs_lin;   /* [n][prsnum][3] at curtime */
  const double *prs_ang;   /* [n][prsnum][3] at curtime */
  const double *obs_ang;   /* [n][obsnum][3] at curtime+step */
  const double *obs_lin;   /* [n][obsnum][3] at curtime+step */
  int stepnum;             /* DEM calls made before this one (stepnum, parmec.cpp:2523; UNSPRING's nsteps) */
} pg_steptab;

/* ======================================================================== */
/* (2) Device-resident session API                                          */
/* ======================================================================== */
typedef struct pg_session pg_session;

/* Numeric form of a session. */
#define PG_FORM_FP64   0   /* plain FP64, bit-exact with the oracle */
#define PG_FORM_MIXED  1   /* FP32 contact geometry and forces, FP64 positions/rotations */

/* Create a session on the current CUDA device and upload the scene.
 * Replaces the buffer set-up of init()/input() (parmec.cpp:2227) plus the
 * per-DEM partitioning_create (partition.ispc:663). */
int pg_session_create(const pg_scene *scene, int form, pg_session **out);

/* Release all device memory of the session. */
int pg_session_destroy(pg_session *s);

/* The curtime == 0 block of dem() (parmec.cpp:2397-2405): euler(0.5*step),
 * full shapes, obstacle velocities at 0.5*step and obstacles(step). */
int pg_session_first_half_step(pg_session *s, double step,
                               const double *obs_ang, const double *obs_lin);

/* invert_inertia (parmec.ispc:90), called by dem() at every DEM call. */
int pg_session_invert_inertia(pg_session *s);

/* Advance tab->nsteps steps of the loop body of dem() (parmec.cpp:2418-2517)
 * with a fixed step (adaptive == 0); returns once the steps finished. */
int pg_session_run(pg_session *s, const pg_steptab *tab, double step);

/* pg_session_run without the final wait: the steps are enqueued on the
 * session stream and the call returns (no counterpart in the reference, whose
 * dem() is synchronous).  'tab' is consumed before the call returns.  The
 * host may prepare its next uploads meanwhile; pg_session_sync waits for the
 * steps.  Sessions with mesh contact on, or stepped by the fused kernel,
 * still read a count back inside the call. */
int pg_session_run_async(pg_session *s, const pg_steptab *tab, double step);

/* Copy the state of particles idx[0..n) (velocities, rotation, position,
 * force, torque) or of springs idx[0..n) (sorted positions: current points,
 * stroke, forces) into the host arrays of 'scene' at the same indices, through
 * one device gather and one small copy.  What output_history reads
 * (output.cpp:5143-5533) without downloading every array. */
int pg_session_download_particles(pg_session *s, pg_scene *scene, const int *idx, int n);
int pg_session_download_springs(pg_session *s, pg_scene *scene, const int *idx, int n);

/* restrain_velocities (restrain.ispc:137) of the scene's restraints: the
 * DEM prologue calls it once after invert_inertia (parmec.cpp:2413).  The
 * per-step restrain_forces runs inside the step. */
int pg_session_restrain_velocities(pg_session *s);

/* The same with adaptive stepping (DEM's 'adaptive', 0 < adaptive <= 1;
 * parmec.cpp:2443-2450, adaptive_timestep parmec.ispc:397-420): step n runs
 * with step0 = the previous step's step1 (the first with 'step0'); its step1
 * is 'adaptive' times the smallest critical step of the particles, estimated
 * on the device from this step's contacts and springs (time_step_task,
 * parmec.ispc:275-383), or step0 when nothing is restrained.  The obstacle
 * rows of 'tab' must be sampled at curtime + step0 of each step, so a caller
 * with time-dependent inputs runs one step per call.  Writes each step's
 * step1 to steps[n] (may be NULL) and waits for the steps to finish.  FP64
 * form, one scene without device excitation; else PG_ERR_UNSUPPORTED. */
int pg_session_run_adaptive(pg_session *s, const pg_steptab *tab, double step0, double adaptive, double *steps);

/* Mesh-mesh contact, an extension with no counterpart in the reference
 * (whose contact detection holds spheres only, partition.ispc:600-646, and
 * returns at once for meshes, condet.ispc:786): every triangle of a MESH
 * particle is swept by a sphere of 'radius', and triangles of different
 * particles closer than 2 * radius touch, with the GRANULAR law of their
 * colours (pg_tritri.cuh states the geometry).  'cell' is the grid cell
 * (at least the largest box of a triangle not flagged in 'big', radius
 * included); big[t] = 1 marks triangles searched against all others.
 * radius = 0 turns it off.  FP64 form, one scene, fixed steps (adaptive
 * stepping returns PG_ERR_UNSUPPORTED while it is on); steps with it run
 * without CUDA graphs. */
int pg_session_mesh_contact(pg_session *s, double radius, double cell, const unsigned char *big);
/* A pool's live extents: the steps cover particles [0, particles), spheres
 * [0, spheres) and triangles [0, triangles) of the session's arrays, whose
 * entries beyond are free (scene id -1).  A serving pool sized for its
 * whole memory budget then costs per step what its admitted scenes hold.
 * The values must not exceed the session's counts; the counts themselves
 * restore the whole arrays.  The next step rebuilds the candidate lists. */
int pg_session_set_live(pg_session *s, int particles, int spheres, int triangles);

/* Triangle pairs whose boxes overlapped in the last step, and those in contact. */
int pg_session_mesh_contact_stats(pg_session *s, int *pairs, int *active);

/* CRITICAL (input.cpp:3034-3154) on the device.  which = 0: per particle
 * (critical_perparticle, parmec.ispc:547-888) from the contacts of the last
 * step and the springs: h, omega, ratio get parnum entries; which = 1: per
 * spring (critical_perspring, parmec.ispc:485-544): sprnum entries, in the
 * session's sorted spring order.  Contact normals are the recorded ones when
 * the session records geometry (pg_session_record_geometry), else the
 * direction from the partner to the sphere centre at the current positions.
 * FP64 form; PG_ERR_UNSUPPORTED for the mixed form. */
int pg_session_critical(pg_session *s, int which, double *h, double *omega, double *ratio);

/* Wait for the session stream; returns the first device error seen. */
int pg_session_sync(pg_session *s);

/* Copy the dynamic state back into the host arrays of 'scene' (the same
 * layout that was uploaded): particles, spheres, triangles, obstacles,
 * nodes and spring state. */
int pg_session_download(pg_session *s, pg_scene *scene);

/* Re-upload every dynamic array from the host (after host edits between DEM calls). */
int pg_session_upload(pg_session *s, const pg_scene *scene);

/* Number of active contact points (master side). */
int pg_session_contact_count(pg_session *s, int *count);

/* Export the active contacts in the canonical order (master particle, then
 * partner code).  code >= 0 is the slave ellipsoid, code < 0 is -(triangle+1).
 * Arrays hold 'cap' entries; *count returns the number written. */
int pg_session_contacts(pg_session *s, int cap, int *count,
                        int *master_particle, int *code,
                        double *point, double *normal, double *depth,
                        double *force, double *state);

/* CUDA stream used by the session (cudaStream_t as void*). */
int pg_session_stream(pg_session *s, void **stream);

/* Number of kernels the last pg_session_run launched (for bench accounting). */
int pg_session_kernel_launches(pg_session *s, long long *count);

/* Set the skin (Verlet margin) used by contact detection, in length units.
 * A negative value selects the automatic choice. */
int pg_session_set_skin(pg_session *s, double skin);

/* Record contact normals and depths as well (for parity exports; costs
 * bandwidth, off by default). */
int pg_session_record_geometry(pg_session *s, int on);

/* Run steps as one captured CUDA graph per step (on, the default) or as
 * individual stream launches (off).  Results are identical. */
int pg_session_use_graph(pg_session *s, int on);

/* Mixed form only: run each step as one cooperatively launched step kernel
 * (scene excitation, sphere and triangle contacts, integration and obstacles
 * between grid barriers), preceded by the cooperative rebuild kernel, which
 * returns at once unless a rebuild is due; 16 steps are captured as one CUDA
 * graph per replay.  Results are bit-identical to the per-phase kernels for
 * any launch shape.  A grid barrier that waits more than 2 s gives PG_ERR_TIMEOUT in
 * the diagnostics instead of hanging.  PG_ERR_UNSUPPORTED in the FP64 form. */
int pg_session_use_fused(pg_session *s, int on);

/* Let the next runs pick the fused kernel's launch shape (threads per block,
 * blocks per SM) by timing the candidates on the session's own first steps;
 * the steps are real steps of the run. */
int pg_session_autotune(pg_session *s, int on);

/* out4 = {threads per block, blocks, 1 if tuned, 1 if running as a graph}. */
int pg_session_fused_config(pg_session *s, int *out4);

/* Page-lock (pin) a host buffer that sessions copy to and from, so that the
 * copies of upload/download run at full link speed (NVLink-C2C on GB300), and
 * release it.  Registering an already registered buffer is PG_OK. */
int pg_host_register(void *ptr, size_t bytes);
int pg_host_unregister(void *ptr);

/* Self-test of the bounded grid barrier used by the cooperative kernels: a
 * small cooperative grid waits at a barrier that cannot complete, gives up
 * after its 2 s limit and records PG_ERR_TIMEOUT; the session stays usable.
 * Returns PG_OK when the timeout was recorded (wait_ms: the kernel's time). */
int pg_session_barrier_selftest(pg_session *s, double *wait_ms);

/* ---- scenes sharing a session -------------------------------------------
 * Every scene has its own grid origin (cells of a common size), its own
 * triangles, an active flag, a local time origin and optionally a base
 * excitation evaluated on the device at t = (global step - start step)*step:
 *   g(t) = g0 + dir * sum_k amp_k * sin(2*pi*freq_k*t + phase_k),  k < ncomp <= 8,
 * stored as PG_EXC_LEN doubles {g0x,g0y,g0z, dirx,diry,dirz, ncomp, 0,
 * amp_0,freq_0,phase_0, ..., amp_7,freq_7,phase_7}.  Scenes never interact,
 * and a scene's arithmetic is the same whichever other scenes share the
 * session. */
#define PG_EXC_LEN 32

/* Candidate-list capacity: kn slots per sphere and kr slave slots per
 * particle (1..96, default 32).  Contact lists restart empty. */
int pg_session_set_capacity(pg_session *s, int kn, int kr);

/* Common grid of every scene: cell size and cells per axis (1..512); the
 * cell tables are reallocated for nscene << (3*bits) cells. */
int pg_session_set_grid(pg_session *s, double cell, const int dim[3]);

/* Scene control: active flag; grid origin (NULL keeps it); excitation
 * record of PG_EXC_LEN doubles (NULL: gravity from the step table);
 * start_step < 0 takes the current global step. */
int pg_session_scene(pg_session *s, int scene, int active, const double origin[3],
                     const double excitation[PG_EXC_LEN], long long start_step);

/* Copy the ranges [p0,p1) particles, [e0,e1) spheres, [t0,t1) triangles,
 * [o0,o1) obstacles of a pooled host scene to the device (range = {p0,p1,e0,
 * e1,t0,t1,o0,o1}); candidate lists of those spheres restart empty. */
int pg_session_upload_range(pg_session *s, const pg_scene *scene, const int range[8]);

/* Copy the same ranges of the dynamic state back to the host scene. */
int pg_session_download_range(pg_session *s, pg_scene *scene, const int range[8]);

/* The motion state of the particle range alone (position, linear and angular
 * velocity rows): what a finished request of a serving pool hands back.  The
 * scene's other host arrays are left as they were. */
int pg_session_download_range_motion(pg_session *s, pg_scene *scene, const int range[8]);

/* Free the same ranges in a pool: their particles, spheres, triangles and
 * obstacles get scene id -1, which every kernel skips, and the spheres'
 * candidate lists restart empty.  Only device scene ids change: the state
 * arrays keep their values until the next upload of the ranges.  No
 * counterpart in the reference, which runs one scene per process. */
int pg_session_release_range(pg_session *s, const int range[8]);

/* Steps the session has run so far. */
int pg_session_global_step(pg_session *s, long long *step);

/* Time kernel groups with CUDA events on the session stream during
 * pg_session_run (on != 0) and reset the accumulators.  Groups: 0 rebuild of
 * candidate lists, 1 contacts, 2 springs, 3 integrate, 4 mesh nodes/faces,
 * 5 obstacles and step tail. */
int pg_session_profile(pg_session *s, int on);

/* Accumulated milliseconds and kernel launches per group (8 entries each). */
int pg_session_profile_read(pg_session *s, double *ms, long long *launches);

/* Diagnostics (16 ints): [0..3] first device error (status, site, index,
 * value; site 1 = candidate list, 3 = slave list, 4 = pairing kind),
 * [4] rebuilds so far, [5] largest candidate count seen, [6] largest slave
 * count, [7] largest triangle candidate count, [12..14] grid cells per axis,
 * [15] Morton bits per axis. */
int pg_session_diagnostics(pg_session *s, int *out16);

/* ======================================================================== */
/* (3) Building blocks on caller-owned device memory                         */
/* ======================================================================== */

/* Morton-ordered cell list of n sphere centres (device arrays x, y, z):
 * replaces partitioning_create (partition.ispc:663).  Cells of size 'cell'
 * from 'origin' with dim[k] cells per axis (1..1024; positions outside are
 * clamped to the border cells).  Writes, to device arrays of n entries, the
 * Morton key of every sphere's cell in ascending order (keys_out) and the
 * sphere indices in that order (order_out; stable, so equal keys keep index
 * order).  Enqueued on 'stream' (a cudaStream_t, or NULL); scratch memory is
 * taken with cudaMallocAsync and released on the same stream. */
int pg_cell_order(const double *x, const double *y, const double *z, int n,
                  const double origin[3], double cell, const int dim[3],
                  unsigned *keys_out, int *order_out, void *stream);

/* pg_cell_order without any device allocation (no counterpart in the
 * reference).  For callers that cannot allocate device memory -- coupling
 * codes whose own pool owns the device memory, and hosts that cannot afford
 * the device synchronisation cudaMalloc/cudaFree may cause.  Scratch lives in
 * a static device array of the library, sized for at most 65,536 spheres
 * (about 0.55 MB, held by every GPU that loads the library until exit);
 * larger n returns PG_ERR_CAPACITY.  Calls share that array: calls that
 * overlap on the GPU race.  A call on a stream that is not capturing looks
 * up the array's address on the current device; a call during stream
 * capture uses the address found by the last such call, so the first call
 * on a device (and the first after a device reset) should come before any
 * stream capture.  Same arguments and results as pg_cell_order. */
int pg_cell_order_static(const double *x, const double *y, const double *z, int n,
                         const double origin[3], double cell, const int dim[3],
                         unsigned *keys_out, int *order_out, void *stream);

/* Library version string. */
const char *pg_version(void);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* PARMEC_GB300_H */
