/* parmec_ispc.h -- drop-in replacement of the ISPC export surface that
 * parmec.cpp links against.
 *
 * Parmec's C++ host includes the headers that ISPC generates from its kernels
 * (objs8/<file>_ispc.h, included at parmec.cpp:46-52, "using namespace ispc"
 * at parmec.cpp:55) and calls the exports below with REAL = double.  This
 * header declares the same functions, with the same names, argument order and
 * meaning, inside namespace ispc and with C linkage, so that parmec.cpp
 * compiles against it unchanged and links against libparmec_gb300.so instead
 * of the ISPC objects.
 *
 * Each function is synchronous, as the ISPC exports are ("launch ... sync"):
 * it copies the host arrays it reads to the device, runs the GPU kernels and
 * copies back the arrays it writes before it returns.  Host memory stays the
 * truth between calls.  The device keeps what the reference keeps behind
 * opaque pointers: the contact lists with their tangential state (owned by
 * the master array of master_alloc) and the spatial grid (partitioning).
 * `ntasks` is accepted and ignored: the GPU picks its own parallelism.
 *
 * Errors: the reference exits through ASSERT (macros.h:68-72) or asserts on
 * unsupported cases.  These functions print the reason and exit(1) by
 * default; pg_compat_exit_on_error(0) makes them record the first error for
 * pg_compat_status() instead and return.
 */
#ifndef PARMEC_ISPC_H
#define PARMEC_ISPC_H

#ifdef __cplusplus
namespace ispc {
extern "C" {
#endif

#define PG_ISPC_CONBUF 8     /* condet.h:29 */
#define PG_ISPC_NSTATE 8     /* condet.h:28 */
#define PG_ISPC_NMAT 3       /* constants.h:33 */
#define PG_ISPC_NIPARAM 7    /* constants.h:37 */

/* master contact points of one particle, a list of blocks (condet.h:33-49);
 * the layout is the reference's, so that code reading the lists compiles.
 * The device holds the contacts; pg_compat_materialize writes them here. */
struct master_conpnt
{
  int master[PG_ISPC_CONBUF];            /* sphere (ellipsoid) index */
  int slave[2][PG_ISPC_CONBUF];          /* partner particle or triangle owner code, partner sphere or -(triangle+1) */
  int color[2][PG_ISPC_CONBUF];
  double point[3][PG_ISPC_CONBUF];
  double normal[3][PG_ISPC_CONBUF];
  double depth[PG_ISPC_CONBUF];
  double force[3][PG_ISPC_CONBUF];
  double kcur[PG_ISPC_CONBUF];
  double ecur[PG_ISPC_CONBUF];
  double state[PG_ISPC_NSTATE][PG_ISPC_CONBUF];
  int size;
  struct master_conpnt *next;
  int lock;
};

/* slave contact points (condet.h:53-64): mirrors of master entries */
struct slave_conpnt
{
  int master[2][PG_ISPC_CONBUF];         /* master particle, master sphere */
  double point[3][PG_ISPC_CONBUF];
  double force[3][PG_ISPC_CONBUF];
  double kcur[PG_ISPC_CONBUF];
  double ecur[PG_ISPC_CONBUF];
  int size;
  struct slave_conpnt *next;
  int lock;
};

/* the spatial grid handle (replaces partition.ispc's kd-tree); opaque */
struct partitioning;

/* ---- memory and cores (parmec.ispc:30-59).  Real and int buffers come
 * from page-locked host memory when a CUDA device is present, so that the
 * per-call copies run at full link speed; else from ordinary aligned memory. */
int ispc_num_cores (void);
double *aligned_real_alloc (int n);
void aligned_real_free (double *ptr);
int *aligned_int_alloc (int n);
void aligned_int_free (int *ptr);

/* ---- contact lists (condet.ispc:703-778): 'old' and its contact state move
 * to the new array; free drops the state */
struct master_conpnt *master_alloc (struct master_conpnt *old, int nold, int size);
void master_free (struct master_conpnt *con, int size);
struct slave_conpnt *slave_alloc (struct slave_conpnt *old, int nold, int size);
void slave_free (struct slave_conpnt *con, int size);

/* ---- spatial grid (partition.ispc:663-774).  create returns NULL when
 * ellnum == 0 (as the reference does); store never overflows (returns 0):
 * the grid is rebuilt inside condet when spheres moved far enough. */
struct partitioning *partitioning_create (int ntasks, int ellnum, double *center[6]);
int partitioning_store (int ntasks, struct partitioning *tree, int ellnum, int ellcol[], int part[],
                        double *center[6], double *radii[3], double *orient[18]);
void partitioning_destroy (struct partitioning *tree);

/* ---- the step (condet.ispc:781, forces.ispc:2130, dynamics.ispc:172) */
void condet (int ntasks, struct partitioning *tree, struct master_conpnt master[],
             int parnum, int ellnum, int ellcol[], int part[], double *center[6],
             double *radii[3], double *orient[18], int trinum,
             int tricol[], int triobs[], double *tri[3][3]);

void forces (int ntasks, struct master_conpnt master[], struct slave_conpnt slave[],
             int parnum, double *angular[6], double *linear[3],
             double *rotation[9], double *position[3], double *inertia[9],
             double *inverse[9], double mass[], double invm[], double obspnt[],
             double obslin[], double obsang[], int parmat[], double *mparam[PG_ISPC_NMAT],
             int pairnum, int pairs[], int ikind[], double *iparam[PG_ISPC_NIPARAM],
             double step, int sprnum, int sprtype[], int unspring[], int sprmap[],
             int *sprpart[2], double *sprpnt[2][6], double *spring[2], int spridx[],
             double *dashpot[2], int dashidx[], double *unload[2], int unidx[],
             double *yield[2], double *sprdir[6], int sprflg[], int sproffset[],
             double sprfric[], double sprkskn[], double *sprsdsp[3], double stroke0[],
             double *stroke[3], double *sprfrc[3], double *lcurve[2],
             int lcidx[], double gravity[3], int trqsprnum, int *trqsprpart[2],
             double *trqzdir0[3], double *trqxdir0[3], double *krpy[3][2],
             int *krpyidx[3], double *drpy[3][2], int *drpyidx[3],
             int trqcone[], double *trqzdir1[3], double *trqxdir1[3],
             double *trqrpy[3], double *trqrpytot[3], double *trqrpyspr[3],
             double *force[3], double *torque[3], double *kact[3], double kmax[],
             double emax[], double *krot[6], int adaptive, int unsprnum, int tsprings[],
             int tspridx[], int msprings[], int mspridx[], double *unlim[2], int unent[],
             int unop[], int unabs[], int nsteps[], int nfreq[], int unaction[],
             int activate[], int actidx[], int stepnum, double time);

void dynamics (int ntasks, struct master_conpnt master[], struct slave_conpnt slave[],
               int parnum, double *angular[6], double *linear[3],
               double *rotation[9], double *position[6],
               double *inertia[9], double *inverse[9],
               double mass[], double invm[], double damping[6],
               double *force[3], double *torque[3],
               int flags[], double step0, double step1);

/* ---- per-particle helpers of dem() (parmec.ispc:90, 388; shapes.ispc:214;
 * obstacles.ispc:28) */
void invert_inertia (int ntasks, int size, double *inertia[9], double *inverse[9], double mass[], double invm[]);
void euler (int ntasks, int parnum, double *angular[6], double *linear[3], double *rotation[9],
            double *position[3], double step);
void shapes (int ntasks, int ellnum, int part[], double *center[6], double *radii[3], double *orient[18],
             int nodnum, double *nodes[6], int nodpart[], int *flags,
             int facnum, int *facnod[3], int factri[], double *tri[3][3],
             double *rotation[9], double *position[6]);
void obstacles (int obsnum, int trirng[], double point[], double angular[], double linear[],
                double *tri[3][3], double step);

/* ---- restraints and adaptive stepping, called by dem() beside the hot
 * path (restrain.ispc:137, 147; parmec.ispc:397-420).  All three run on the
 * device with host arrays copied in and out. */
void restrain_velocities (int ntasks, int rstnum, int rstpart[], double *rstlin[9], double *rstang[9],
                          double *linear[3], double *angular[6], double *rotation[9]);
void restrain_forces (int ntasks, int rstnum, int rstpart[], double *rstlin[9], double *rstang[9],
                      double *force[3], double *torque[3]);
double adaptive_timestep (int ntasks, int parnum, double mass[], double *inertia[9], double *kact[3],
                          double kmax[], double emax[], double *krot[6], double step, double adaptive);

/* ---- the setup-time queries input.cpp calls (EQM input.cpp:2378, CRITICAL
 * input.cpp:3064, 3097, 3133), on the device. */
/* eqm (parmec.ispc:423): equivalent point mass of part1 at point1 and part2
 * (or -1: ground) at point2 along direction (zero length: the smallest
 * eigenvalue direction); reads position[3..5] (reference positions) */
double eqm (int part1, double *point1, int part2, double *point2, double *direction,
            double *inverse[9], double invm[], double *position[3]);
/* critical_perspring (parmec.ispc:485): per-spring critical step hcri,
 * circular frequency ocri and damping ratio rcri; particles are read up to
 * the largest index the springs name */
void critical_perspring (int sprnum, int *sprpart[2], double *sprpnt[2][6], double *sprdir[6],
                         double *spring[2], int spridx[], double *dashpot[2], int dashidx[],
                         double *inverse[9], double invm[], double *position[3],
                         double hcri[], double ocri[], double rcri[]);
/* critical_perparticle (parmec.ispc:860): per-particle critical step, frequency
 * and ratio from the contacts that condet()/forces() hold for this master
 * array and from the springs; kact, kmax, emax and krot receive the terms.
 * Returns the smallest step (the reference leaves its return value unset). */
double critical_perparticle (int ntasks, struct master_conpnt master[], struct slave_conpnt slave[],
                             int parnum, double mass[], double *inertia[9], double invm[],
                             double *inverse[9], double *rotation[9], double *position[6],
                             int sprnum, int sprflg[], int *sprpart[2], double *sprpnt[2][6],
                             double *sprdir[6], double *spring[2], int spridx[], double *dashpot[2],
                             int dashidx[], double *kact[3], double kmax[], double emax[],
                             double *krot[6], double hcri[], double ocri[], double rcri[]);

/* ---- GB300 additions (not in the reference) */
int pg_compat_status (void);               /* first error since the last call (PG_ERR_*), then cleared */
void pg_compat_exit_on_error (int on);     /* 1 (default): print and exit(1) like ASSERT; 0: record */
void pg_compat_set_bits (int compat);      /* PG_COMPAT_* defect switches; default EXPMAP | TRIEDGE */
void pg_compat_set_skin (double skin);     /* candidate-list skin; 0: 0.3 * smallest radius */
long long pg_compat_kernel_launches (void);/* GPU kernels launched by the functions above */
/* write the device contacts into the reference's list layout (master and,
 * when given, slave arrays of parnum entries); returns the contact count */
int pg_compat_materialize (struct master_conpnt *master, struct slave_conpnt *slave, int parnum);

#ifdef __cplusplus
} /* extern "C" */
} /* namespace ispc */
#endif

#endif
