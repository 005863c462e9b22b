// pg_state.h -- device-resident scene of one session.
//
// Layout in HBM: structure of arrays, one contiguous array per vector
// component (as the reference's host buffers, parmec.cpp:61-285), so a warp
// reading component k of 32 consecutive particles reads 256 contiguous bytes.
// Contact candidate lists are slot-major ([slot][sphere]) so that slot k of a
// warp's 32 spheres is one coalesced segment.
#pragma once
#include <cstdint>

#define PG_EXC_LEN 32       // doubles per excitation record: g0[3], dir[3], ncomp, pad, 8 x (amp, freq, phase)

struct PgDev
{
  int parnum, ellnum, trinum, obsnum, nodnum, facnum, sprnum, pairnum, prsnum;
  int compat;
  int form;                 // PG_FORM_FP64 / PG_FORM_MIXED

  // ---- particles (parmec.cpp:95-114)
  double *angular[6], *linear[3], *rotation[9], *position[6];
  double *inertia[9], *inverse[9], *mass, *invm, *force[3], *torque[3];
  int *flags, *parmat;
  unsigned char *piso;      // 1: inertia j*I and inverse (1/j)*I with +0 off the diagonal (FP64 form)
  int *pell;                // particle -> its sphere, or -1

  // ---- spheres (parmec.cpp:86-93)
  double *center[6], *radii[3];
  int *ellcol, *part;

  // ---- triangles and obstacles
  double *tri[9];           // tri[3*vertex + coord]
  int *tricol, *triobs;
  int *trirng;              // [2*obsnum]
  int *triown;              // triangle -> moving obstacle index, or -1
  double *obspnt, *obsang, *obslin;   // [3*obsnum]

  // ---- surface pairing
  int *pairs, *ikind;
  double *iparam[7];

  // ---- mesh nodes and faces
  double *nodes[6];
  int *nodpart;
  int *facnod[3], *factri;

  // ---- springs (parmec.cpp:151-178)
  int *sprtype, *unspring, *sprpart[2];
  double *sprpnt[12];       // sprpnt[6*side + k]
  double *spring[2]; int *spridx;
  double *dashpot[2]; int *dashidx;
  double *unload[2]; int *unidx;
  double *yield[2], *sprdir[6];
  int *sprflg, *sproffset;
  double *sprfric, *sprkskn, *sprsdsp[3], *stroke0, *stroke[3], *sprfrc[3];
  double *lcurve[2]; int *lcidx;
  double *spr_out[9];       // per spring: frc[3], trq_j[3], trq_k[3]
  int *sev_first;           // [parnum+1] CSR of spring force events per particle
  int4 *sev;                // (type | (long run + 1) << 1, begin, end, first): type 0 = j-run (+=), 1 = k-run (-=)
  int4 *sbig;               // [nbig] the long runs
  double *sbig_sum;         // [nbig][6] their force and torque sums
  double *sbig_grp;         // [nbig][32][12] group partials of the long-run sums
  int nbig;

  // ---- adaptive time step (parmec.ispc:275-420, forces.ispc:453-596, 1248-1345)
  double *hs;               // [3]: step0, step1, factor (null: fixed step, from the kernel arguments)
  double *hrec;             // [table rows] step1 of each step of a call
  unsigned long long *hmin; // smallest critical step of the particles, as the bits of a non-negative double
  double *akact[3], *akrot[6], *akmax, *aemax;   // [parnum] stiffness terms (k_contacts: master side only)
  double *sad[17];          // [sprnum] |z| (3), |stiffness|, |damping|, krot of the j arm (6) and of the k arm (6)
  double *sbig_ad;          // [nbig][11] long-run partials: kact (3), krot (6), kmax, emax

  // ---- restraints (restrain.ispc:30-133), CSR per particle in input order
  int rstnum;
  int *rst_first;           // [parnum+1]
  int *rst_list;            // restraint indices
  double *rstlin[9], *rstang[9];   // [rstnum] three orthonormal directions each (zero rows unused)

  // ---- torsion springs (trqspr_task, forces.ispc:1415-2057), sorted by (part0, part1)
  int trqsprnum;
  int *trqsprpart[2];
  double *trqzdir0[3], *trqxdir0[3];
  double *krpy[3][2]; int *krpyidx[3];
  double *drpy[3][2]; int *drpyidx[3];
  int *trqcone;
  double *trqzdir1[3], *trqxdir1[3], *trqrpy[3], *trqrpytot[3], *trqrpyspr[3];
  double *tq_out[3];        // per torsion spring: torque in the global frame
  double *tq_k[3];          // per torsion spring: adaptive krot diagonal terms
  int *tev_first;           // [parnum+1] CSR of torsion torque flush events per particle
  int4 *tev;                // (type, begin, end, first) as sev, without long-run chunking

  // ---- prescribed body forces (prescribe_body_forces, parmec.cpp:2202-2224)
  int pbfnum;
  int *pbf_slot;            // [parnum] record of the particle, or -1
  double *pbfout[6], *pbfin[6];   // [pbfnum] outer (added) and inner (exported) force and torque

  // ---- spring failure rules (unspring_task, forces.ispc:2058-2127); spring
  // lists hold sorted positions
  int unsprnum;
  int *u_t, *u_tidx, *u_m, *u_midx, *u_a, *u_aidx;
  double *unlim[2];
  int *unent, *unop, *unabs, *unsteps, *nfreq, *unaction;
  int *ustep;               // stepnum of the running DEM call (from the step table)

  // ---- prescribed motion
  int *prs_first;           // [parnum+1] CSR of prescriptions per particle
  int *prs_list;            // prescription indices in input order
  int *prslin, *prsang, *linkind, *angkind;

  // ---- per-step host tables on the device
  double *t_curtime, *t_gravity, *t_damping, *t_prs_lin, *t_prs_ang, *t_obs_ang, *t_obs_lin;
  int tab_prs_stride, tab_obs_stride;   // rows: prsnum*3, obsnum*3 (at least 3)
  int *stepno;              // device step counter (row of the tables)

  // ---- contact candidates (Verlet lists), master side, slot-major
  int kn;                   // slots per sphere
  int estride;              // sphere stride of the slot-major arrays ([slot][estride]); the sphere
                            // capacity, which a pool's live view keeps while its ellnum shrinks
  int *ncnt;                // [ellnum]
  int *ncode;               // [kn][ellnum]: sphere j >= 0, or -(triangle+1)
  unsigned char *nflag;     // [kn][ellnum]: contact active
  double *nstate[3];        // [kn][ellnum]: tangential spring state
  double *nfrc[3];          // [kn][ellnum]: contact force on the master
  double *npnt[3];          // [kn][ellnum]: contact point
  double *nen;              // [kn][ellnum]: normal damping of the pair, damper*2*sqrt(kn*m) (FP64 session)
  double *nnrm[3], *ndep;   // normal and depth (depth: parity exports only)
  int *cwork, *cwork_n;     // [kn][ellnum] work queue of the FP64 contact evaluation, and its length
  int record_geometry;
  double *fm[3], *tm[3];    // [parnum] master-side partial force and torque sums
  int kr;                   // (unused: slave lists have no per-particle limit)
  // slave lists, CSR over particles: the entries that name particle p as
  // partner are rref[soff[p] .. soff[p+1]), each the candidate-entry index
  // slot*ellnum + sphere, ordered by (master particle, slot)
  int *rcnt;                // [parnum] entries per particle
  int *soff;                // [parnum+1]
  int *rref;                // = sval[0] after the entry sort
  int *eorder;              // [ellnum] spheres in particle order (stable)
  int *eoff;                // [ellnum+1] first entry of each sphere of eorder; eoff[ellnum] = total
  unsigned *skey[2];        // [kn*ellnum] entry sort: partner particle (0xffffffff: none)
  int *sval[2];             // [kn*ellnum] entry sort: entry index
  unsigned *shist;          // entry-sort tile histograms
  int *smeta;               // [5]: entries, tiles, histogram length, scan tiles of it, longest slave list
  unsigned *sbs;            // scan block sums
  int sbits;                // bits of the entry-sort keys

  // ---- rebuild machinery
  int *rebuild;             // 1 when the candidate lists must be rebuilt
  int *obs_done;            // [1]: blocks of the step's obstacle update that finished (the last runs the tail)
  int *err;                 // [4]: first device error (PG_ERR_*), site, index, value; 0 when fine
  unsigned *gbar;           // [4]: grid barrier of the fused step kernel: arrivals, generation, abort
  int *stats;               // [8]: rebuilds, max candidates, max slave entries, max triangles per sphere
  double skin, cell, half_skin_sq;
  double org[3];
  int dim[3], bits, keybits;   // cells per axis, Morton bits per axis, bits of (scene, cell) keys
  double *cref[3];          // sphere centres at the last rebuild
  float4 *cfs;              // [ellnum] float centre and radius of the sphere at each sorted position (rebuild)
  int *pfs;                 // [ellnum] particle of the sphere at each sorted position (rebuild)
  unsigned *ekey;           // [ellnum] cell key of each sphere at the last rebuild, in sphere order
  double *tref[9];          // triangle vertices at the last rebuild
  unsigned *keys[2];        // radix-sort ping-pong buffers
  int *vals[2];
  unsigned *hist;           // radix-sort block histograms
  int nsortblocks;
  int *cstart, *cend;       // [2^(3*bits)] cell ranges in sorted order
  int *ncnt_new;            // scratch candidate lists of a rebuild
  int *ncode_new;
  float *tbox;              // [6][trinum] triangle AABBs at rebuild (float, widened)

  // ---- mesh-mesh contact (extension, pg_meshcontact.cu): per-particle
  // force and torque sums of this step's triangle contacts, added after
  // gravity by the force sums when tt_on
  int tt_on;
  double *ttF[3], *ttT[3];

  // ---- independent scenes in one session (batching / serving pool)
  int nscene;
  int *pscene;              // [parnum] scene of each particle
  int *escene;              // [ellnum] scene of each sphere
  int *tscene;              // [trinum] scene of each triangle
  int *oscene;              // [obsnum] scene of each obstacle
  int *sactive;             // [nscene] 1 when the scene steps
  int *stbeg, *stend;       // [nscene] triangle range of each scene
  double *sorg[3];          // [nscene] grid origin of each scene (common cell and dims)
  int *sexc_on;             // [nscene] 1: gravity from the device excitation, 0: from the step table
  double *sexc;             // [nscene][PG_EXC_LEN] excitation records (see pg_session_scene)
  double *sgrav;            // [nscene][3] gravity of this step (k_excite)
  long long *sstart;        // [nscene] global step at which the scene's local time is 0
  long long *gstep;         // global step counter

  // ---- mixed form (PG_FORM_MIXED): compensated FP32 pairs for positions,
  // linear velocities, rotations and radii; FP32 for everything else
  float *xh[3], *xl[3], *vh[3], *vl[3], *Lh[9], *Ll[9];
  float *Om[3], *om[3];     // referential and spatial angular velocity
  float *rh, *rl;           // sphere radius pairs
  float *mass_f, *invm_f, *J_f[9], *I_f[9];
  float *F_f[3], *T_f[3];
  float *nstate_f[3], *nfrc_f[3], *narm_f[3];   // per candidate entry; arm = point - slave position
  float *fm_f[3], *tm_f[3];
  int *twork;               // [ellnum] spheres with triangle candidates this step
  int *tcnt;                // [2] length of twork, blocks of the triangle pass done
  float *iparam_f[7];       // [pairnum] surface pair parameters in FP32
  float *sgrav_f;           // [nscene][3] this step's scene gravity in FP32 (written with sgrav)
  float *damp_f;            // [6] this step's damping row in FP32
  float *jiso, *iiso;       // [parnum] j and 1/j when the inertia is j*I (isotropic), else 0
  float *cref_f[3];         // [ellnum] sphere centres at the last rebuild (hi parts)
  float half_skin_sq_f;
};
