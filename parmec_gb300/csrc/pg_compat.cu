// pg_compat.cu -- the ISPC export surface that parmec.cpp calls
// (include/parmec_ispc.h), on the GPU.
//
// parmec.cpp's dem() (parmec.cpp:2386-2517) calls euler, shapes, obstacles,
// invert_inertia, partitioning_*, condet, forces and dynamics on host SoA
// buffers it owns, and runs its own host code between them (prescribed
// motion, joints, restraints, output).  So every function here:
//   1. copies the host arrays it reads into a device mirror,
//   2. runs the same kernels as the session (pg_step.cu, pg_rebuild.cu,
//      pg_sort.cu),
//   3. copies back the arrays it writes and returns when the device is done.
// Host memory is the truth between calls.  The device keeps only what the
// reference keeps behind its own opaque pointers: the contact candidate
// lists with their tangential state (the reference's master_conpnt lists,
// owned here by the master array of master_alloc) and the spatial grid.
//
// The split of the work differs from the reference where the result cannot
// tell: condet() brings the candidate lists up to date (the rebuild gated by
// displacement), and forces() evaluates every candidate's geometry, the
// contact creation/removal rule and the force in one pass (k_contacts).  The
// unmodified loop calls condet() and forces() back to back on the same
// positions, so the contact set and forces are the reference's.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>
#include "pg_state.h"
#include "pg_launch.h"
#include "../../include/parmec_gb300.h"
#include "../../include/parmec_ispc.h"

namespace ispc {
struct partitioning { int ellnum; };
}

namespace {

using ispc::master_conpnt;
using ispc::slave_conpnt;

struct Compat
{
  bool init = false;
  cudaStream_t st = nullptr;
  PgDev d{};                                  // device mirrors and contact state
  std::unordered_map<void *, size_t> cap;     // elements allocated behind each PgDev pointer field
  const void *owner = nullptr;                // master array that owns the contact state
  bool lists = false;                         // contact lists exist for (P, E, T) below
  int P = -1, E = -1, T = -1;
  int obs_known = 0;                          // obstacles of the last obstacles() call
  int obs_rows = 0;                           // obstacle velocity rows the triangles of the last condet() use
  double skin = 0.0;                          // 0: 0.3 * smallest radius
  int bits = PG_COMPAT_EXPMAP | PG_COMPAT_TRIEDGE;
  int status = PG_OK;
  int exit_on_error = 1;
  long long launches = 0;
  const char *fn = "";                        // entry point running (for messages)
  std::vector<int> h_part, h_ellcol, h_triobs, h_tricol;   // of the last condet(), for materialize
  double *hs = nullptr;                       // adaptive stepping: step0, step1, factor (view().hs when used)
  double *crit_ke = nullptr;                  // CRITICAL: per-spring largest slope and damping
  double *crit_h = nullptr, *crit_o = nullptr, *crit_r = nullptr;   // CRITICAL outputs
  PgDev eqd{};                                // eqm: the two particles' rows
  double *eq_pts = nullptr, *eq_out = nullptr;
};

Compat G;
std::mutex M;                                 // the exports are called from one thread; serialise anyway
std::mutex Mpin;
std::unordered_set<void *> pinned;

void fail(int code, const char *what)
{
  if (G.status == PG_OK) G.status = code;
  std::fprintf(stderr, "parmec_gb300 drop-in: %s: %s\n", G.fn, what);
  if (G.exit_on_error) std::exit(1);
}

bool cuda_ok(cudaError_t e, const char *what)
{
  if (e == cudaSuccess) return true;
  char msg[256];
  std::snprintf(msg, sizeof msg, "%s: %s", what, cudaGetErrorString(e));
  fail(PG_ERR_CUDA, msg);
  return false;
}

template <typename T>
bool grow(T *&f, size_t n)
{
  if (n == 0) n = 1;
  size_t &c = G.cap[(void *)&f];
  if (f && c >= n) return true;
  if (f)
  {
    if (!cuda_ok(cudaStreamSynchronize(G.st), "cudaStreamSynchronize")) return false;
    cudaFree(f);
    f = nullptr;
  }
  c = 0;
  void *q = nullptr;
  if (!cuda_ok(cudaMalloc(&q, n * sizeof(T)), "cudaMalloc")) return false;
  if (!cuda_ok(cudaMemsetAsync(q, 0, n * sizeof(T), G.st), "cudaMemsetAsync")) return false;
  f = (T *)q;
  c = n;
  return true;
}

// grow and keep the first 'keep' elements
template <typename T>
bool grow_keep(T *&f, size_t n, size_t keep)
{
  size_t &c = G.cap[(void *)&f];
  if (f && c >= n) return true;
  T *old = f;
  const size_t oldc = c;
  f = nullptr;
  c = 0;
  if (!grow(f, n)) return false;
  if (old)
  {
    keep = std::min(keep, oldc);
    if (keep && !cuda_ok(cudaMemcpyAsync(f, old, keep * sizeof(T), cudaMemcpyDeviceToDevice, G.st), "copy")) return false;
    if (!cuda_ok(cudaStreamSynchronize(G.st), "cudaStreamSynchronize")) return false;
    cudaFree(old);
  }
  return true;
}

template <typename T>
bool up(T *&f, const T *h, size_t n)
{
  if (!grow(f, n)) return false;
  if (n && h) return cuda_ok(cudaMemcpyAsync(f, h, n * sizeof(T), cudaMemcpyHostToDevice, G.st), "host to device copy");
  return true;
}

template <typename T>
bool down(T *h, const T *f, size_t n)
{
  if (n && h && f) return cuda_ok(cudaMemcpyAsync(h, f, n * sizeof(T), cudaMemcpyDeviceToHost, G.st), "device to host copy");
  return true;
}

template <typename T>
bool zeros(T *&f, size_t n)
{
  if (!grow(f, n)) return false;
  return cuda_ok(cudaMemsetAsync(f, 0, std::max<size_t>(n, 1) * sizeof(T), G.st), "cudaMemsetAsync");
}

// wait for the device and turn a device-side error record into a failure
bool finish(const char *fn)
{
  if (!cuda_ok(cudaGetLastError(), fn)) return false;
  int err[4] = {0, 0, 0, 0};
  if (!cuda_ok(cudaMemcpyAsync(err, G.d.err, sizeof err, cudaMemcpyDeviceToHost, G.st), fn)) return false;
  if (!cuda_ok(cudaStreamSynchronize(G.st), fn)) return false;
  if (err[0] != 0)
  {
    int z[4] = {0, 0, 0, 0};
    cudaMemcpy(G.d.err, z, sizeof z, cudaMemcpyHostToDevice);
    char msg[160];
    std::snprintf(msg, sizeof msg, "%s: device error %d at site %d (index %d, value %d)", fn, err[0], err[1], err[2], err[3]);
    fail(err[0], msg);
    return false;
  }
  return true;
}

bool ready()
{
  if (G.init) return true;
  if (!cuda_ok(cudaStreamCreateWithFlags(&G.st, cudaStreamNonBlocking), "no CUDA device")) return false;
  PgDev &d = G.d;
  d.form = PG_FORM_FP64;
  d.nscene = 1;
  d.kn = 32;
  d.kr = 32;
  d.record_geometry = 1;
  d.tab_prs_stride = 3;
  d.tab_obs_stride = 3;
  const int one = 1;
  bool ok = grow(d.sactive, 1) && up(d.sactive, &one, 1) && grow(d.stbeg, 1) && grow(d.stend, 1) &&
            grow(d.sexc_on, 1) && grow(d.sexc, PG_EXC_LEN) && grow(d.sgrav, 3) && grow(d.sstart, 1) &&
            grow(d.gstep, 1) && grow(d.stepno, 1) && grow(d.rebuild, 1) && grow(d.err, 4) && grow(d.stats, 8) &&
            grow(d.t_curtime, 1) && grow(d.t_gravity, 3) && grow(d.t_damping, 6) && grow(d.t_prs_lin, 3) &&
            grow(d.t_prs_ang, 3) && grow(d.t_obs_ang, 3) && grow(d.t_obs_lin, 3);
  for (int k = 0; ok && k < 3; k ++) ok = grow(d.sorg[k], 1);
  if (!ok || !cuda_ok(cudaStreamSynchronize(G.st), "set-up")) return false;
  G.init = true;
  return true;
}

// candidate-list storage for kn slots per sphere and kr slave slots per
// particle (grown in place: entry k of sphere i sits at k*E + i)
bool slot_arrays(size_t keep_slots)
{
  PgDev &d = G.d;
  const size_t E = std::max(d.ellnum, 1), P = std::max(d.parnum, 1);
  const size_t n = (size_t)d.kn * E;
  bool ok = grow_keep(d.ncode, n, keep_slots) && grow_keep(d.nflag, n, keep_slots) && grow_keep(d.ndep, n, keep_slots) &&
            grow(d.cwork, n) && grow(d.cwork_n, 1);
  for (int k = 0; ok && k < 3; k ++)
    ok = grow_keep(d.nstate[k], n, keep_slots) && grow_keep(d.nfrc[k], n, keep_slots) &&
         grow_keep(d.npnt[k], n, keep_slots) && grow_keep(d.nnrm[k], n, keep_slots);
  // slave-list entries (at most kn per sphere) and their sort and scan scratch
  for (int k = 0; ok && k < 2; k ++) ok = grow(d.skey[k], n) && grow(d.sval[k], n);
  const int nb = pg_sort_blocks((int)n);
  const int sb = std::max(pg_scan_blocks(256 * nb), std::max(pg_scan_blocks((int)E + 1), pg_scan_blocks((int)P + 1)));
  ok = ok && grow(d.shist, 256 * (size_t)nb) && grow(d.sbs, (size_t)sb);
  d.rref = d.sval[pg_sort_passes_exact(d.sbits) & 1];
  return ok;
}

// (re)start the contact state for P particles, E spheres and T triangles
bool restart_lists(int P, int E, int T)
{
  PgDev &d = G.d;
  d.parnum = P; d.ellnum = E; d.trinum = T;
  d.estride = E;
  d.sbits = pg_rebuild_entry_bits(P);
  bool ok = zeros(d.ncnt, E) && zeros(d.rcnt, P) && grow(d.soff, (size_t)P + 1) && grow(d.eorder, E) &&
            grow(d.eoff, (size_t)E + 1) && grow(d.smeta, 5) && grow(d.gbar, 4) && slot_arrays(0);
  for (int k = 0; ok && k < 3; k ++) ok = grow(d.cref[k], E) && grow(d.fm[k], P) && grow(d.tm[k], P);
  ok = ok && grow(d.cfs, E) && grow(d.pfs, E) && grow(d.ekey, E);
  for (int k = 0; ok && k < 9; k ++) ok = grow(d.tref[k], T);
  ok = ok && grow(d.tbox, 6 * (size_t)std::max(T, 1));
  for (int k = 0; ok && k < 2; k ++) ok = grow(d.keys[k], E) && grow(d.vals[k], E);
  d.nsortblocks = pg_sort_blocks(E);
  ok = ok && grow(d.hist, 256 * (size_t)d.nsortblocks);
  // no previous sort: the free-entry key makes the range clear skip every
  // sphere, and the cell tables of an earlier scene are cleared in full
  ok = ok && cuda_ok(cudaMemsetAsync(d.keys[0], 0xff, (size_t)std::max(E, 1) * sizeof(unsigned), G.st), "memset");
  for (int *t : {d.cstart, d.cend})
    if (ok && t) ok = cuda_ok(cudaMemsetAsync(t, 0, G.cap[t == d.cstart ? (void *)&d.cstart : (void *)&d.cend] *
                                                    sizeof(int), G.st), "memset");
  ok = ok && zeros(d.escene, E) && zeros(d.pscene, P) && zeros(d.tscene, T);
  d.skin = G.skin;
  G.P = P; G.E = E; G.T = T;
  G.lists = ok;
  return ok;
}

// grid for the current sphere centres (host copies) and the skin
bool set_grid(const double *const cx[3], const double *r, int E)
{
  PgDev &d = G.d;
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300}, rmax = 0.0, rmin = 1e300;
  for (int e = 0; e < E; e ++)
  {
    for (int k = 0; k < 3; k ++)
    {
      const double c = cx[k][e];
      if (c == c) { lo[k] = std::min(lo[k], c); hi[k] = std::max(hi[k], c); }
    }
    rmax = std::max(rmax, r[e]);
    rmin = std::min(rmin, r[e]);
  }
  if (!(rmax > 0.0)) { rmax = rmin = 1e-3; }
  double ext[3];
  for (int k = 0; k < 3; k ++)
  {
    if (!(hi[k] >= lo[k])) { lo[k] = 0.0; hi[k] = 0.0; }
    ext[k] = std::max(hi[k] - lo[k], 1e-300);
  }
  pg_rebuild_grid_params(d, ext, rmax, rmin);
  if (pg_rebuild_sort_bits(d) > 32) { fail(PG_ERR_ARGUMENT, "condet: grid keys exceed 32 bits"); return false; }
  for (int k = 0; k < 3; k ++)
  {
    const double o = lo[k] - 4.0 * d.cell;
    if (!up(d.sorg[k], &o, 1)) return false;
  }
  const size_t cells = (size_t)1 << (3 * d.bits);
  return grow(d.cstart, cells) && grow(d.cend, cells);
}

// the view of the mirrors that the step kernels get
PgDev view()
{
  PgDev v = G.d;
  v.compat = G.bits;
  return v;
}

} // namespace

namespace ispc {
extern "C" {

// ---------------------------------------------------------------- memory (parmec.ispc:30-59)
int ispc_num_cores(void)
{
  unsigned n = std::thread::hardware_concurrency();
  return n ? (int)n : 1;
}

static void *host_alloc(size_t bytes)
{
  if (bytes == 0) bytes = 8;
  void *p = nullptr;
  if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) == cudaSuccess)
  {
    std::lock_guard<std::mutex> g(Mpin);
    pinned.insert(p);
  }
  else
  {
    cudaGetLastError();
    p = nullptr;
    if (posix_memalign(&p, 64, bytes) != 0) p = nullptr;
  }
  if (p) std::memset(p, 0, bytes);
  return p;
}

static void host_free(void *p)
{
  if (!p) return;
  {
    std::lock_guard<std::mutex> g(Mpin);
    auto it = pinned.find(p);
    if (it != pinned.end())
    {
      pinned.erase(it);
      cudaFreeHost(p);
      return;
    }
  }
  std::free(p);
}

double *aligned_real_alloc(int n) { return (double *)host_alloc((size_t)std::max(n, 0) * sizeof(double)); }
void aligned_real_free(double *ptr) { host_free(ptr); }
int *aligned_int_alloc(int n) { return (int *)host_alloc((size_t)std::max(n, 0) * sizeof(int)); }
void aligned_int_free(int *ptr) { host_free(ptr); }

// ---------------------------------------------------------------- contact lists (condet.ispc:703-778)
master_conpnt *master_alloc(master_conpnt *old, int nold, int size)
{
  std::lock_guard<std::mutex> g(M);
  master_conpnt *con = new master_conpnt[std::max(size, 1)]();
  if (nold && old)
  {
    std::memcpy((void *)con, (const void *)old, (size_t)nold * sizeof(master_conpnt));
    delete[] old;
  }
  for (int i = nold; i < size; i ++) { con[i].size = 0; con[i].next = nullptr; con[i].lock = -1; }
  if (old && G.owner == old) G.owner = con;
  return con;
}

void master_free(master_conpnt *con, int size)
{
  std::lock_guard<std::mutex> g(M);
  if (!con) return;
  for (int i = 0; i < size; i ++)
    for (master_conpnt *p = con[i].next; p;)
    {
      master_conpnt *n = p->next;
      delete p;
      p = n;
    }
  if (G.owner == con) { G.owner = nullptr; G.lists = false; }
  delete[] con;
}

slave_conpnt *slave_alloc(slave_conpnt *old, int nold, int size)
{
  slave_conpnt *con = new slave_conpnt[std::max(size, 1)]();
  if (nold && old)
  {
    std::memcpy((void *)con, (const void *)old, (size_t)nold * sizeof(slave_conpnt));
    delete[] old;
  }
  for (int i = 0; i < size; i ++) { con[i].size = 0; con[i].next = nullptr; con[i].lock = -1; }
  return con;
}

void slave_free(slave_conpnt *con, int size)
{
  if (!con) return;
  for (int i = 0; i < size; i ++)
    for (slave_conpnt *p = con[i].next; p;)
    {
      slave_conpnt *n = p->next;
      delete p;
      p = n;
    }
  delete[] con;
}

// ---------------------------------------------------------------- grid handle (partition.ispc:663-774)
partitioning *partitioning_create(int, int ellnum, double *[6])
{
  if (ellnum == 0) return nullptr;
  partitioning *t = new partitioning;
  t->ellnum = ellnum;
  return t;
}

int partitioning_store(int, partitioning *tree, int ellnum, int[], int[], double *[6], double *[3], double *[18])
{
  if (tree) tree->ellnum = ellnum;
  return 0;
}

void partitioning_destroy(partitioning *tree) { delete tree; }

// ---------------------------------------------------------------- invert_inertia (parmec.ispc:90)
void invert_inertia(int, int size, double *inertia[9], double *inverse[9], double mass[], double invm[])
{
  std::lock_guard<std::mutex> g(M);
  G.fn = "invert_inertia";
  if (size <= 0 || !ready()) return;
  PgDev &d = G.d;
  const size_t P = size;
  bool ok = true;
  for (int k = 0; ok && k < 9; k ++) ok = up(d.inertia[k], inertia[k], P) && grow(d.inverse[k], P);
  ok = ok && up(d.mass, mass, P) && grow(d.invm, P);
  if (!ok) return;
  PgDev v = view();
  v.parnum = size;
  pg_launch_invert(v, G.st);
  G.launches += 1;
  for (int k = 0; ok && k < 9; k ++) ok = down(inverse[k], d.inverse[k], P);
  if (ok && down(invm, d.invm, P)) finish("invert_inertia");
}

// ---------------------------------------------------------------- euler (parmec.ispc:388)
void euler(int, int parnum, double *angular[6], double *linear[3], double *rotation[9], double *position[3], double step)
{
  std::lock_guard<std::mutex> g(M);
  G.fn = "euler";
  if (parnum <= 0 || !ready()) return;
  PgDev &d = G.d;
  const size_t P = parnum;
  bool ok = true;
  for (int k = 0; ok && k < 3; k ++) ok = up(d.angular[k], angular[k], P) && grow(d.angular[3+k], P);
  for (int k = 0; ok && k < 3; k ++) ok = up(d.linear[k], linear[k], P) && up(d.position[k], position[k], P);
  for (int k = 0; ok && k < 9; k ++) ok = up(d.rotation[k], rotation[k], P);
  if (!ok) return;
  PgDev v = view();
  v.parnum = parnum;
  pg_launch_euler(v, G.st, step);
  G.launches += 1;
  for (int k = 0; ok && k < 3; k ++) ok = down(angular[3+k], d.angular[3+k], P) && down(position[k], d.position[k], P);
  for (int k = 0; ok && k < 9; k ++) ok = down(rotation[k], d.rotation[k], P);
  if (ok) finish("euler");
}

// ---------------------------------------------------------------- shapes (shapes.ispc:214)
void shapes(int, int ellnum, int part[], double *center[6], double *[3], double *[18],
            int nodnum, double *nodes[6], int nodpart[], int *flags,
            int facnum, int *facnod[3], int factri[], double *tri[3][3],
            double *rotation[9], double *position[6])
{
  std::lock_guard<std::mutex> g(M);
  G.fn = "shapes";
  if ((ellnum <= 0 && nodnum <= 0) || !ready()) return;
  PgDev &d = G.d;
  // the particles the spheres and nodes belong to
  int P = 0, T = 0;
  for (int e = 0; e < ellnum; e ++) P = std::max(P, part[e] + 1);
  for (int n = 0; n < nodnum; n ++) P = std::max(P, nodpart[n] + 1);
  for (int f = 0; f < facnum; f ++) T = std::max(T, factri[f] + 1);
  bool ok = true;
  for (int k = 0; ok && k < 9; k ++) ok = up(d.rotation[k], rotation[k], P);
  for (int k = 0; ok && k < 6; k ++) ok = up(d.position[k], position[k], P);
  if (ellnum > 0)
  {
    for (int k = 0; ok && k < 6; k ++) ok = up(d.center[k], center[k], ellnum);
    ok = ok && up(d.part, part, ellnum);
  }
  if (nodnum > 0)
  {
    for (int k = 0; ok && k < 6; k ++) ok = up(d.nodes[k], nodes[k], nodnum);
    ok = ok && up(d.nodpart, nodpart, nodnum);
    if (flags) ok = ok && up(d.flags, flags, P);
  }
  const bool fac = facnum > 0 && T > 0;
  if (fac)
  {
    for (int k = 0; ok && k < 3; k ++) ok = up(d.facnod[k], facnod[k], facnum);
    ok = ok && up(d.factri, factri, facnum);
    for (int a = 0; ok && a < 3; a ++)
      for (int c = 0; ok && c < 3; c ++) ok = up(d.tri[3*a+c], tri[a][c], T);
  }
  if (!ok) return;
  // the view is taken after the uploads: an upload may (re)allocate a mirror
  PgDev v = view();
  v.parnum = P;
  v.ellnum = std::max(ellnum, 0);
  v.nodnum = std::max(nodnum, 0);
  v.facnum = 0;
  v.trinum = 0;
  pg_launch_shapes(v, G.st, flags != nullptr);              // spheres, then nodes
  G.launches += (v.ellnum ? 1 : 0) + (v.nodnum ? 1 : 0);
  if (fac)
  {
    // faces after nodes; the vertices serve as their own reference (the
    // session's displacement flag is unused: condet() decides rebuilds)
    PgDev f = v;
    f.ellnum = 0;
    f.nodnum = 0;
    f.facnum = facnum;
    f.trinum = T;
    for (int k = 0; k < 9; k ++) f.tref[k] = d.tri[k];
    pg_launch_shapes(f, G.st, false);
    G.launches += 1;
  }
  for (int k = 0; ok && k < 3 && ellnum > 0; k ++) ok = down(center[k], d.center[k], ellnum);
  for (int k = 0; ok && k < 3 && nodnum > 0; k ++) ok = down(nodes[k], d.nodes[k], nodnum);
  for (int a = 0; ok && a < 3 && fac; a ++)
    for (int c = 0; ok && c < 3; c ++) ok = down(tri[a][c], d.tri[3*a+c], T);
  if (ok) finish("shapes");
}

// ---------------------------------------------------------------- obstacles (obstacles.ispc:28)
void obstacles(int obsnum, int trirng[], double point[], double angular[], double linear[], double *tri[3][3], double step)
{
  std::lock_guard<std::mutex> g(M);
  G.fn = "obstacles";
  if (obsnum <= 0 || !ready()) return;
  G.obs_known = obsnum;
  PgDev &d = G.d;
  int T = 0;
  for (int o = 0; o < obsnum; o ++) T = std::max(T, trirng[2*o+1]);
  std::vector<int> own(std::max(T, 1), -1);
  for (int o = 0; o < obsnum; o ++)
    for (int t = std::max(trirng[2*o], 0); t < trirng[2*o+1]; t ++) own[t] = o;
  bool ok = up(d.obspnt, point, 3 * (size_t)obsnum) && up(d.obsang, angular, 3 * (size_t)obsnum) &&
            up(d.obslin, linear, 3 * (size_t)obsnum) && zeros(d.oscene, obsnum);
  if (T > 0)
  {
    for (int a = 0; ok && a < 3; a ++)
      for (int c = 0; ok && c < 3; c ++) ok = up(d.tri[3*a+c], tri[a][c], T);
    ok = ok && up(d.triown, own.data(), T) && zeros(d.tscene, std::max(T, G.T));
  }
  if (!ok) return;
  // the view is taken after the uploads: an upload may (re)allocate a mirror
  PgDev v = view();
  v.obsnum = obsnum;
  v.trinum = T;
  v.ellnum = 0;                               // no rebuild flag from here: condet() decides
  // the vertices serve as their own reference (the displacement test is unused)
  for (int k = 0; k < 9; k ++) v.tref[k] = d.tri[k];
  pg_launch_obstacles_state(v, G.st, step);
  G.launches += (T ? 1 : 0) + 1;
  for (int a = 0; ok && a < 3 && T > 0; a ++)
    for (int c = 0; ok && c < 3; c ++) ok = down(tri[a][c], d.tri[3*a+c], T);
  ok = ok && down(point, d.obspnt, 3 * (size_t)obsnum);
  if (ok) finish("obstacles");
}

// ---------------------------------------------------------------- condet (condet.ispc:781)
void condet(int, partitioning *tree, master_conpnt master[], int parnum, int ellnum, int ellcol[], int part[],
            double *center[6], double *radii[3], double *[18], int trinum, int tricol[], int triobs[], double *tri[3][3])
{
  if (tree == nullptr) return;                // condet.ispc:786
  std::lock_guard<std::mutex> g(M);
  G.fn = "condet";
  if (ellnum <= 0 || parnum <= 0 || !ready()) return;
  PgDev &d = G.d;
  // spheres only, one per particle (the reference asserts on ellipsoids, condet.ispc:33-47)
  std::vector<int> pell(parnum, -1);
  for (int e = 0; e < ellnum; e ++)
  {
    const int p = part[e];
    if (p < 0 || p >= parnum) { fail(PG_ERR_ARGUMENT, "condet: sphere of no particle"); return; }
    if (!(radii[1][e] < 0.0)) { fail(PG_ERR_UNSUPPORTED, "condet: ellipsoids are not supported"); return; }
    if (pell[p] >= 0) { fail(PG_ERR_UNSUPPORTED, "condet: a particle with more than one sphere"); return; }
    pell[p] = e;
  }
  const int T = std::max(trinum, 0);
  const bool restart = !G.lists || G.owner != (const void *)master || G.P != parnum || G.E != ellnum || G.T != T;
  if (restart && !restart_lists(parnum, ellnum, T)) return;
  G.owner = master;
  d.parnum = parnum; d.ellnum = ellnum; d.trinum = T;
  d.estride = ellnum;
  bool ok = true;
  for (int k = 0; ok && k < 3; k ++) ok = up(d.center[k], center[k], ellnum);
  std::vector<int> ord(ellnum);
  for (int e = 0; e < ellnum; e ++) ord[e] = e;
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return part[a] < part[b]; });
  ok = ok && up(d.radii[0], radii[0], ellnum) && up(d.part, part, ellnum) && up(d.ellcol, ellcol, ellnum) &&
       up(d.pell, pell.data(), parnum) && up(d.eorder, ord.data(), ellnum) &&
       cuda_ok(cudaStreamSynchronize(G.st), "condet");           // ord is a local
  for (int a = 0; ok && a < 3; a ++)
    for (int c = 0; ok && c < 3; c ++) ok = up(d.tri[3*a+c], T ? tri[a][c] : nullptr, T);
  ok = ok && up(d.tricol, T ? tricol : nullptr, T) && up(d.triobs, T ? triobs : nullptr, T);
  const int zero = 0;
  ok = ok && up(d.stbeg, &zero, 1) && up(d.stend, &T, 1);
  if (!ok) return;
  G.h_part.assign(part, part + ellnum);
  G.h_ellcol.assign(ellcol, ellcol + ellnum);
  G.h_triobs.assign(triobs, triobs + T);
  G.h_tricol.assign(tricol, tricol + T);
  int rows = 0;                               // obstacles the triangles name
  for (int t = 0; t < T; t ++)
    if (triobs[t] <= -2) rows = std::max(rows, -triobs[t] - 2 + 1);
  G.obs_rows = rows;

  // is a rebuild due?
  int due = 1;
  if (restart) ok = up(d.rebuild, &due, 1);
  else
  {
    ok = zeros(d.rebuild, 1);
    PgDev v = view();
    if (d.half_skin_sq <= 0.0) ok = ok && up(d.rebuild, &due, 1);
    pg_launch_rebuild_gate(v, G.st);
    G.launches += 1;
    ok = ok && down(&due, d.rebuild, 1) && cuda_ok(cudaStreamSynchronize(G.st), "condet");
  }
  if (!ok) return;
  if (due)
  {
    if (!set_grid(center, radii[0], ellnum)) return;
    for (int attempt = 0; attempt < 4; attempt ++)
    {
      const int one = 1;
      if (!up(d.rebuild, &one, 1)) return;
      PgDev v = view();
      pg_launch_rebuild(v, G.st);
      G.launches += pg_rebuild_kernel_count(v);
      int err[4] = {0, 0, 0, 0}, stats[8];
      if (!down(err, d.err, 4) || !down(stats, d.stats, 8) || !cuda_ok(cudaStreamSynchronize(G.st), "condet")) return;
      if (err[0] != PG_ERR_CAPACITY) break;
      // a list overflowed: more slots (contacts beyond the old capacity restart their state)
      const int z[4] = {0, 0, 0, 0};
      if (!up(d.err, z, 4)) return;
      const int kn = std::min(96, std::max(d.kn, stats[1] + 8));
      if (kn == d.kn)
      {
        char msg[200];
        std::snprintf(msg, sizeof msg, "more than 96 contact candidates (site %d, index %d, count %d; "
                      "largest list %d)", err[1], err[2], err[3], stats[1]);
        fail(PG_ERR_CAPACITY, msg);
        return;
      }
      const size_t keep = (size_t)d.kn * ellnum;
      d.kn = kn;
      if (!slot_arrays(keep)) return;
    }
  }
  finish("condet");
}

// ---------------------------------------------------------------- forces (forces.ispc:2130)
void forces(int, master_conpnt master[], slave_conpnt[], int parnum, double *angular[6], double *linear[3],
            double *rotation[9], double *position[3], double *inertia[9], double *inverse[9], double mass[], double invm[],
            double obspnt[], double obslin[], double obsang[], int[], double *[PG_ISPC_NMAT],
            int pairnum, int pairs[], int ikind[], double *iparam[PG_ISPC_NIPARAM],
            double step, int sprnum, int sprtype[], int unspring[], int sprmap[],
            int *sprpart[2], double *sprpnt[2][6], double *spring[2], int spridx[],
            double *dashpot[2], int dashidx[], double *unload[2], int unidx[],
            double *yield[2], double *sprdir[6], int sprflg[], int sproffset[],
            double sprfric[], double sprkskn[], double *sprsdsp[3], double stroke0[],
            double *stroke[3], double *sprfrc[3], double *lcurve[2],
            int lcidx[], double gravity[3], int trqsprnum, int *trqsprpart[2],
            double *trqzdir0[3], double *trqxdir0[3], double *krpy[3][2], int *krpyidx[3], double *drpy[3][2],
            int *drpyidx[3], int trqcone[], double *trqzdir1[3], double *trqxdir1[3], double *trqrpy[3],
            double *trqrpytot[3], double *trqrpyspr[3],
            double *force[3], double *torque[3], double *kact[3], double kmax[],
            double emax[], double *krot[6], int adaptive, int unsprnum, int tsprings[],
            int tspridx[], int msprings[], int mspridx[], double *unlim[2], int unent[], int unop[], int unabs[],
            int nsteps[], int nfreq[], int unaction[], int activate[], int actidx[], int stepnum, double time)
{
  std::lock_guard<std::mutex> g(M);
  G.fn = "forces";
  if (parnum <= 0 || !ready()) return;

  if (unsprnum > 0 && (sprnum <= 0 || !sprmap)) { fail(PG_ERR_ARGUMENT, "forces: UNSPRING needs the springs and sprmap"); return; }
  if (adaptive && (!kact || !kmax || !emax || !krot))
  {
    fail(PG_ERR_ARGUMENT, "forces: adaptive stepping needs kact, kmax, emax and krot");
    return;
  }
  PgDev &d = G.d;
  const size_t P = parnum, S = std::max(sprnum, 0);
  const bool contacts = G.lists && G.owner == (const void *)master && G.P == parnum && G.E > 0;
  bool ok = true;
  for (int k = 0; ok && k < 3; k ++)
    ok = up(d.angular[3+k], angular[3+k], P) && up(d.linear[k], linear[k], P) && up(d.position[k], position[k], P);
  ok = ok && up(d.mass, mass, P) && up(d.invm, invm, P) && zeros(d.pscene, P);
  for (int k = 0; ok && k < 3; k ++) ok = grow(d.force[k], P) && grow(d.torque[k], P);   // written by the sums
  ok = ok && up(d.pairs, pairs, 2 * (size_t)pairnum) && up(d.ikind, ikind, (size_t)pairnum);
  for (int k = 0; ok && k < PG_ISPC_NIPARAM; k ++) ok = up(d.iparam[k], iparam[k], (size_t)pairnum);
  // obstacle velocity rows the contact triangles use (never past the obstacles known)
  // (with the reference's index defect a triangle reads the next obstacle's
  // row, so one more row when that many obstacles exist)
  int rows = G.obs_rows;
  if ((G.bits & PG_COMPAT_OBSIDX) && G.obs_known > rows) rows += 1;
  if (G.obs_known > 0) rows = std::min(rows, G.obs_known);
  if (rows > 0)
    ok = ok && up(d.obspnt, obspnt, 3 * (size_t)rows) && up(d.obslin, obslin, 3 * (size_t)rows) &&
         up(d.obsang, obsang, 3 * (size_t)rows);
  // gravity of this step (read_gravity_and_damping on the host) and the time for springs
  ok = ok && up(d.sgrav, gravity, 3) && up(d.t_curtime, &time, 1) && zeros(d.stepno, 1) && zeros(d.sexc_on, 1);
  if (S || adaptive)
    for (int k = 0; ok && k < 9; k ++) ok = up(d.rotation[k], rotation[k], P);
  if (adaptive)
  {
    // stiffness terms (forces.ispc:453-596, 1248-1345) and the step for the kernels
    for (int k = 0; ok && k < 3; k ++) ok = grow(d.akact[k], P);
    for (int k = 0; ok && k < 6; k ++) ok = grow(d.akrot[k], P);
    ok = ok && grow(d.akmax, P) && grow(d.aemax, P);
    for (int k = 0; ok && k < 17; k ++) ok = grow(d.sad[k], S);
    const double h3[3] = {step, step, 1.0};
    ok = ok && up(G.hs, h3, 3);
  }
  if (S)
  {
    for (int k = 0; ok && k < 9; k ++) ok = up(d.inertia[k], inertia[k], P) && up(d.inverse[k], inverse[k], P);
    for (int k = 0; ok && k < 3; k ++) ok = up(d.position[3+k], position[3+k], P);
    ok = ok && up(d.sprtype, sprtype, S) && up(d.unspring, unspring, S);
    for (int k = 0; ok && k < 2; k ++) ok = up(d.sprpart[k], sprpart[k], S);
    for (int a = 0; ok && a < 2; a ++)
      for (int k = 0; ok && k < 6; k ++) ok = up(d.sprpnt[6*a+k], sprpnt[a][k], S);
    const size_t ns = spridx ? spridx[S] : 0, nd = dashidx ? dashidx[S] : 0, nu = unidx ? unidx[S] : 0;
    for (int k = 0; ok && k < 2; k ++)
      ok = up(d.spring[k], spring[k], ns) && up(d.dashpot[k], dashpot[k], nd) && up(d.unload[k], unload[k], nu) &&
           up(d.yield[k], yield[k], S);
    ok = ok && up(d.spridx, spridx, S + 1) && up(d.dashidx, dashidx, S + 1) && up(d.unidx, unidx, S + 1);
    for (int k = 0; ok && k < 6; k ++) ok = up(d.sprdir[k], sprdir[k], S);
    ok = ok && up(d.sprflg, sprflg, S) && up(d.sproffset, sproffset, S) && up(d.sprfric, sprfric, S) &&
         up(d.sprkskn, sprkskn, S) && up(d.stroke0, stroke0, S);
    for (int k = 0; ok && k < 3; k ++)
      ok = up(d.sprsdsp[k], sprsdsp[k], S) && up(d.stroke[k], stroke[k], S) && up(d.sprfrc[k], sprfrc[k], S);
    int nlc = 0;
    for (size_t i = 0; sproffset && i < S; i ++) nlc = std::max(nlc, sproffset[i] + 1);
    for (int i = 0; unaction && i < unsprnum; i ++) nlc = std::max(nlc, unaction[i] + 1);
    const size_t nl = (nlc > 0 && lcidx) ? (size_t)lcidx[nlc] : 0;
    ok = ok && up(d.lcidx, nlc > 0 ? lcidx : nullptr, (size_t)nlc + 1);
    for (int k = 0; ok && k < 2; k ++) ok = up(d.lcurve[k], nlc > 0 ? lcurve[k] : nullptr, nl);
    for (int k = 0; ok && k < 9; k ++) ok = grow(d.spr_out[k], S);
    std::vector<int> first;
    std::vector<int4> ev, big;
    pg_spring_events(parnum, (int)S, sprpart[0], sprpart[1], first, ev, big);
    ok = ok && up(d.sev_first, first.data(), P + 1) && up(d.sev, ev.data(), ev.size()) &&
         up(d.sbig, big.data(), big.size()) && grow(d.sbig_sum, 6 * std::max<size_t>(1, big.size())) &&
         grow(d.sbig_grp, 32 * 12 * std::max<size_t>(1, big.size()));
    if (adaptive) ok = ok && grow(d.sbig_ad, 11 * std::max<size_t>(1, big.size()));
    d.nbig = (int)big.size();
  }
  const int Q = std::max(trqsprnum, 0);
  if (Q)
  {
    // torsion springs: tables, directions, state and their flush events
    if (!(S || adaptive)) for (int k = 0; ok && k < 9; k ++) ok = up(d.rotation[k], rotation[k], P);
    for (int k = 0; ok && k < 9; k ++) ok = up(d.inverse[k], inverse[k], P);
    for (int a = 0; ok && a < 2; a ++) ok = up(d.trqsprpart[a], trqsprpart[a], (size_t)Q);
    for (int c = 0; ok && c < 3; c ++)
      ok = up(d.trqzdir0[c], trqzdir0[c], Q) && up(d.trqxdir0[c], trqxdir0[c], Q) &&
           up(d.trqzdir1[c], trqzdir1[c], Q) && up(d.trqxdir1[c], trqxdir1[c], Q) && up(d.trqrpy[c], trqrpy[c], Q) &&
           up(d.trqrpytot[c], trqrpytot[c], Q) && up(d.trqrpyspr[c], trqrpyspr[c], Q) && grow(d.tq_out[c], Q) &&
           (!adaptive || grow(d.tq_k[c], Q));
    for (int o = 0; ok && o < 3; o ++)
    {
      ok = up(d.krpyidx[o], krpyidx[o], (size_t)Q + 1) && up(d.drpyidx[o], drpyidx[o], (size_t)Q + 1);
      for (int c = 0; ok && c < 2; c ++)
        ok = up(d.krpy[o][c], krpy[o][c], (size_t)krpyidx[o][Q]) && up(d.drpy[o][c], drpy[o][c], (size_t)drpyidx[o][Q]);
    }
    ok = ok && up(d.trqcone, trqcone, (size_t)Q);
    std::vector<int> first;
    std::vector<int4> ev, big;
    pg_spring_events(parnum, Q, trqsprpart[0], trqsprpart[1], first, ev, big);
    for (auto &e : ev) e.x &= 1;               // torsion runs are summed whole
    ok = ok && up(d.tev_first, first.data(), P + 1) && up(d.tev, ev.data(), ev.size());
  }
  const int U = S ? std::max(unsprnum, 0) : 0;
  if (U)
  {
    // spring failure rules, spring ids mapped to sorted positions
    auto mapped = [&](const int *ids, const int *idx, int *&dl, int *&di) -> bool {
      const int n = idx[U];
      std::vector<int> pos(std::max(1, n));
      for (int j = 0; j < n; j ++)
      {
        if (ids[j] < 0 || ids[j] >= sprnum) { fail(PG_ERR_ARGUMENT, "UNSPRING spring index out of range"); return false; }
        pos[j] = sprmap[ids[j]];
      }
      return up(dl, pos.data(), pos.size()) && up(di, idx, (size_t)U + 1);
    };
    ok = ok && mapped(tsprings, tspridx, d.u_t, d.u_tidx) && mapped(msprings, mspridx, d.u_m, d.u_midx) &&
         mapped(activate, actidx, d.u_a, d.u_aidx);
    for (int k = 0; ok && k < 2; k ++) ok = up(d.unlim[k], unlim[k], U);
    ok = ok && up(d.unent, unent, U) && up(d.unop, unop, U) && up(d.unabs, unabs, U) && up(d.unsteps, nsteps, U) &&
         up(d.nfreq, nfreq, U) && up(d.unaction, unaction, U) && up(d.ustep, &stepnum, 1);
  }
  if (!ok) return;
  PgDev v = view();
  v.parnum = parnum;
  v.sprnum = (int)S;
  v.pairnum = pairnum;
  v.obsnum = rows;
  v.prsnum = 0;
  if (!contacts) { v.ellnum = 0; v.pell = nullptr; }
  if (adaptive) v.hs = G.hs;
  v.unsprnum = U;
  v.trqsprnum = Q;
  if (!adaptive) for (int c = 0; c < 3; c ++) v.tq_k[c] = nullptr;
  pg_launch_contacts(v, G.st, step);
  pg_launch_springs(v, G.st, step);
  if (S) pg_launch_spring_runs(v, G.st);
  if (Q) { pg_launch_torsion(v, G.st, step); G.launches += 1; }
  if (U) { pg_launch_unspring(v, G.st); G.launches += 1; }
  if (adaptive) pg_launch_force_sums_adapt(v, G.st);
  else pg_launch_force_sums(v, G.st);
  G.launches += pg_contacts_kernel_count(v) + (S ? 1 : 0) + (S && d.nbig ? (adaptive ? 4 : 2) : 0) + 1;
  for (int k = 0; ok && k < 3; k ++) ok = down(force[k], d.force[k], P) && down(torque[k], d.torque[k], P);
  if (adaptive)
  {
    for (int k = 0; ok && k < 3; k ++) ok = down(kact[k], d.akact[k], P);
    for (int k = 0; ok && k < 6; k ++) ok = down(krot[k], d.akrot[k], P);
    ok = ok && down(kmax, d.akmax, P) && down(emax, d.aemax, P);
  }
  if (S)
  {
    for (int a = 0; ok && a < 2; a ++)
      for (int k = 0; ok && k < 3; k ++) ok = down(sprpnt[a][k], d.sprpnt[6*a+k], S);
    for (int k = 0; ok && k < 3; k ++)
      ok = down(sprdir[k], d.sprdir[k], S) && down(stroke[k], d.stroke[k], S) && down(sprfrc[k], d.sprfrc[k], S) &&
           down(sprsdsp[k], d.sprsdsp[k], S);
    for (int k = 0; ok && k < 2; k ++) ok = down(yield[k], d.yield[k], S);
    ok = ok && down(unspring, d.unspring, S) && down(sprflg, d.sprflg, S);
    if (U) ok = ok && down(nfreq, d.nfreq, U);
  }
  for (int c = 0; ok && Q && c < 3; c ++)
    ok = down(trqzdir1[c], d.trqzdir1[c], Q) && down(trqxdir1[c], d.trqxdir1[c], Q) && down(trqrpy[c], d.trqrpy[c], Q) &&
         down(trqrpytot[c], d.trqrpytot[c], Q) && down(trqrpyspr[c], d.trqrpyspr[c], Q);
  if (!ok) return;
  // zero_force_torque_kmax (forces.ispc) also clears kmax and emax
  if (!adaptive && kmax) std::memset(kmax, 0, P * sizeof(double));
  if (!adaptive && emax) std::memset(emax, 0, P * sizeof(double));
  finish("forces");
}

// ---------------------------------------------------------------- dynamics (dynamics.ispc:172)
void dynamics(int, master_conpnt[], slave_conpnt[], int parnum, double *angular[6], double *linear[3],
              double *rotation[9], double *position[6], double *inertia[9], double *inverse[9],
              double mass[], double invm[], double damping[6], double *force[3], double *torque[3],
              int flags[], double step0, double step1)
{
  std::lock_guard<std::mutex> g(M);
  G.fn = "dynamics";
  if (parnum <= 0 || !ready()) return;
  PgDev &d = G.d;
  const size_t P = parnum;
  bool ok = true;
  for (int k = 0; ok && k < 6; k ++) ok = up(d.angular[k], angular[k], P);
  for (int k = 0; ok && k < 3; k ++)
    ok = up(d.linear[k], linear[k], P) && up(d.position[k], position[k], P) && up(d.force[k], force[k], P) &&
         up(d.torque[k], torque[k], P);
  for (int k = 0; ok && k < 9; k ++)
    ok = up(d.rotation[k], rotation[k], P) && up(d.inertia[k], inertia[k], P) && up(d.inverse[k], inverse[k], P);
  ok = ok && up(d.mass, mass, P) && up(d.invm, invm, P) && up(d.flags, flags, P) && zeros(d.pscene, P) &&
       up(d.t_damping, damping, 6) && zeros(d.stepno, 1);
  if (!ok) return;
  PgDev v = view();
  v.parnum = parnum;
  v.prsnum = 0;
  v.sprnum = 0;
  v.pell = nullptr;                           // the dynamics mode reads no sphere data
  pg_launch_dynamics(v, G.st, step0, step1);
  G.launches += 1;
  for (int k = 0; ok && k < 6; k ++) ok = down(angular[k], d.angular[k], P);
  for (int k = 0; ok && k < 3; k ++)
    ok = down(linear[k], d.linear[k], P) && down(position[k], d.position[k], P) && down(force[k], d.force[k], P) &&
         down(torque[k], d.torque[k], P);
  for (int k = 0; ok && k < 9; k ++) ok = down(rotation[k], d.rotation[k], P);
  if (ok) finish("dynamics");
}

// ---------------------------------------------------------------- outside the hot path
// restraints of one call as per-particle lists in input order, on the device
static bool upload_restraints(int parnum, int rstnum, const int rstpart[], double *rstlin[9], double *rstang[9])
{
  PgDev &d = G.d;
  const size_t P = parnum, R = rstnum;
  std::vector<int> first(P + 1, 0), list(std::max<size_t>(1, R));
  for (size_t q = 0; q < R; q ++)
  {
    if (rstpart[q] < 0 || rstpart[q] >= parnum) { fail(PG_ERR_ARGUMENT, "restraint particle out of range"); return false; }
    first[rstpart[q] + 1] ++;
  }
  for (size_t p = 0; p < P; p ++) first[p+1] += first[p];
  std::vector<int> fill(first.begin(), first.end() - 1);
  for (size_t q = 0; q < R; q ++) list[fill[rstpart[q]] ++] = (int)q;
  bool ok = up(d.rst_first, first.data(), P + 1) && up(d.rst_list, list.data(), list.size());
  for (int k = 0; ok && k < 9; k ++) ok = up(d.rstlin[k], rstlin[k], R) && up(d.rstang[k], rstang[k], R);
  return ok;
}

// ---------------------------------------------------------------- restrain (restrain.ispc:137-154)
void restrain_velocities(int, int rstnum, int rstpart[], double *rstlin[9], double *rstang[9], double *linear[3],
                         double *angular[6], double *rotation[9])
{
  std::lock_guard<std::mutex> g(M);
  G.fn = "restrain_velocities";
  if (rstnum <= 0 || !ready()) return;
  int parnum = 0;
  for (int q = 0; q < rstnum; q ++) parnum = std::max(parnum, rstpart[q] + 1);
  PgDev &d = G.d;
  const size_t P = parnum;
  bool ok = upload_restraints(parnum, rstnum, rstpart, rstlin, rstang);
  for (int k = 0; ok && k < 3; k ++) ok = up(d.linear[k], linear[k], P);
  for (int k = 0; ok && k < 6; k ++) ok = up(d.angular[k], angular[k], P);
  for (int k = 0; ok && k < 9; k ++) ok = up(d.rotation[k], rotation[k], P);
  if (!ok) return;
  PgDev v = view();
  v.parnum = parnum;
  v.rstnum = rstnum;
  pg_launch_restrain_velocities(v, G.st);
  G.launches += 1;
  for (int k = 0; ok && k < 3; k ++) ok = down(linear[k], d.linear[k], P);
  for (int k = 0; ok && k < 6; k ++) ok = down(angular[k], d.angular[k], P);
  if (ok) finish("restrain_velocities");
}

void restrain_forces(int, int rstnum, int rstpart[], double *rstlin[9], double *rstang[9], double *force[3],
                     double *torque[3])
{
  std::lock_guard<std::mutex> g(M);
  G.fn = "restrain_forces";
  if (rstnum <= 0 || !ready()) return;
  int parnum = 0;
  for (int q = 0; q < rstnum; q ++) parnum = std::max(parnum, rstpart[q] + 1);
  PgDev &d = G.d;
  const size_t P = parnum;
  bool ok = upload_restraints(parnum, rstnum, rstpart, rstlin, rstang);
  for (int k = 0; ok && k < 3; k ++) ok = up(d.force[k], force[k], P) && up(d.torque[k], torque[k], P);
  if (!ok) return;
  PgDev v = view();
  v.parnum = parnum;
  v.rstnum = rstnum;
  pg_launch_restrain_forces(v, G.st);
  G.launches += 1;
  for (int k = 0; ok && k < 3; k ++) ok = down(force[k], d.force[k], P) && down(torque[k], d.torque[k], P);
  if (ok) finish("restrain_forces");
}

// ---------------------------------------------------------------- adaptive_timestep (parmec.ispc:397-420)
double adaptive_timestep(int, int parnum, double mass[], double *inertia[9], double *kact[3], double kmax[],
                         double emax[], double *krot[6], double curstep, double adaptive)
{
  std::lock_guard<std::mutex> g(M);
  G.fn = "adaptive_timestep";
  if (parnum <= 0 || !ready()) return curstep;
  PgDev &d = G.d;
  const size_t P = parnum;
  bool ok = up(d.mass, mass, P) && zeros(d.pscene, P);
  for (int k = 0; ok && k < 9; k ++) ok = up(d.inertia[k], inertia[k], P);
  for (int k = 0; ok && k < 3; k ++) ok = up(d.akact[k], kact[k], P);
  for (int k = 0; ok && k < 6; k ++) ok = up(d.akrot[k], krot[k], P);
  ok = ok && up(d.akmax, kmax, P) && up(d.aemax, emax, P);
  const double h3[3] = {curstep, curstep, adaptive};
  const unsigned long long big = 0x7fefffffffffffffull;
  ok = ok && up(G.hs, h3, 3) && up(d.hmin, &big, 1);
  if (!ok) return curstep;
  PgDev v = view();
  v.parnum = parnum;
  v.hs = G.hs;
  pg_launch_adapt_step(v, G.st);
  G.launches += 2;
  double h1 = curstep;
  if (!down(&h1, G.hs + 1, 1) || !finish("adaptive_timestep")) return curstep;
  return h1;
}

// ---------------------------------------------------------------- eqm (parmec.ispc:423-482)
// The equivalent point mass of the EQM command (input.cpp:2336-2381): the
// two particles' rows go to the device and the same eqm as the springs'
// critical damping evaluates it.
double eqm(int part1, double *point1, int part2, double *point2, double *direction, double *inverse[9],
           double invm[], double *position[3])
{
  std::lock_guard<std::mutex> g(M);
  G.fn = "eqm";
  if (part1 < 0 || !point1 || !inverse || !invm || !position || !ready()) return 0.0;
  PgDev &e = G.eqd;
  const int n = part2 >= 0 ? 2 : 1;
  const int rows[2] = {part1, part2};
  double inv[9][2], im[2], pos[3][2], pts[9];
  for (int r = 0; r < n; r ++)
  {
    for (int k = 0; k < 9; k ++) inv[k][r] = inverse[k][rows[r]];
    im[r] = invm[rows[r]];
    for (int k = 0; k < 3; k ++) pos[k][r] = position[3+k][rows[r]];
  }
  for (int k = 0; k < 3; k ++)
  {
    pts[k] = point1[k];
    pts[3+k] = part2 >= 0 && point2 ? point2[k] : 0.0;
    pts[6+k] = direction ? direction[k] : 0.0;
  }
  bool ok = up(e.invm, im, n) && up(G.eq_pts, pts, 9) && grow(G.eq_out, 1);
  for (int k = 0; ok && k < 9; k ++) ok = up(e.inverse[k], inv[k], n);
  for (int k = 0; ok && k < 3; k ++) ok = up(e.position[3+k], pos[k], n);
  if (!ok) return 0.0;
  pg_launch_eqm_one(e, G.st, part2, G.eq_pts, G.eq_out);
  G.launches += 1;
  double out = 0.0;
  if (!down(&out, G.eq_out, 1) || !finish("eqm")) return 0.0;
  return out;
}

// upload the spring arrays CRITICAL reads; P particles' rows of inverse,
// invm and the reference positions (for eqm)
static bool upload_critical_springs(int P, int sprnum, int *sprpart[2], double *sprpnt[2][6], double *sprdir[6],
                                    double *spring[2], int spridx[], double *dashpot[2], int dashidx[],
                                    double *inverse[9], double invm[], double *position[], int sprflg[])
{
  PgDev &d = G.d;
  const size_t S = sprnum;
  bool ok = up(d.invm, invm, P);
  for (int k = 0; ok && k < 9; k ++) ok = up(d.inverse[k], inverse[k], P);
  for (int k = 0; ok && k < 3; k ++) ok = up(d.position[3+k], position[3+k], P);
  for (int k = 0; ok && k < 2; k ++) ok = up(d.sprpart[k], sprpart[k], S);
  for (int a = 0; ok && a < 2; a ++)
    for (int k = 0; ok && k < 6; k ++) ok = up(d.sprpnt[6*a+k], sprpnt[a][k], S);
  for (int k = 0; ok && k < 3; k ++) ok = up(d.sprdir[k], sprdir[k], S);
  const size_t ns = spridx ? spridx[S] : 0, nd = dashidx ? dashidx[S] : 0;
  for (int k = 0; ok && k < 2; k ++) ok = up(d.spring[k], spring[k], ns) && up(d.dashpot[k], dashpot[k], nd);
  ok = ok && up(d.spridx, spridx, S + 1) && up(d.dashidx, dashidx, S + 1);
  if (sprflg) ok = ok && up(d.sprflg, sprflg, S);
  return ok;
}

// ---------------------------------------------------------------- critical_perspring (parmec.ispc:485-544)
void critical_perspring(int sprnum, int *sprpart[2], double *sprpnt[2][6], double *sprdir[6], double *spring[2],
                        int spridx[], double *dashpot[2], int dashidx[], double *inverse[9], double invm[],
                        double *position[3], double hcri[], double ocri[], double rcri[])
{
  std::lock_guard<std::mutex> g(M);
  G.fn = "critical_perspring";
  if (sprnum <= 0 || !ready()) return;
  // the call names no particle count: the rows up to the largest spring end
  int P = 1;
  for (int j = 0; j < sprnum; j ++) P = std::max(P, std::max(sprpart[0][j], sprpart[1][j]) + 1);
  const size_t S = sprnum;
  bool ok = upload_critical_springs(P, sprnum, sprpart, sprpnt, sprdir, spring, spridx, dashpot, dashidx, inverse,
                                    invm, position, nullptr) &&
            grow(G.crit_h, S) && grow(G.crit_o, S) && grow(G.crit_r, S);
  if (!ok) return;
  PgDev v = view();
  v.sprnum = sprnum;
  pg_launch_critical_perspring(v, G.st, G.crit_h, G.crit_o, G.crit_r);
  G.launches += 1;
  ok = down(hcri, G.crit_h, S) && down(ocri, G.crit_o, S) && down(rcri, G.crit_r, S);
  if (ok) finish("critical_perspring");
}

// ---------------------------------------------------------------- critical_perparticle (parmec.ispc:860-888)
// The contact terms come from the device contact lists that condet() and
// forces() keep for this master array.  Returns the smallest particle step
// (the reference declares a return value it never sets).
double critical_perparticle(int, master_conpnt master[], slave_conpnt[], int parnum, double mass[],
                            double *inertia[9], double invm[], double *inverse[9], double *rotation[9],
                            double *position[6], int sprnum, int sprflg[], int *sprpart[2], double *sprpnt[2][6],
                            double *sprdir[6], double *spring[2], int spridx[], double *dashpot[2], int dashidx[],
                            double *kact[3], double kmax[], double emax[], double *krot[6], double hcri[],
                            double ocri[], double rcri[])
{
  std::lock_guard<std::mutex> g(M);
  G.fn = "critical_perparticle";
  const double big = 1.7976931348623157e308;
  if (parnum <= 0 || !ready()) return big;
  PgDev &d = G.d;
  const size_t P = parnum, S = std::max(sprnum, 0);
  const bool contacts = G.lists && G.owner == (const void *)master && G.P == parnum && G.E > 0;
  bool ok = up(d.mass, mass, P) && up(d.invm, invm, P);
  for (int k = 0; ok && k < 9; k ++) ok = up(d.inertia[k], inertia[k], P) && up(d.rotation[k], rotation[k], P);
  for (int k = 0; ok && k < 3; k ++) ok = up(d.position[k], position[k], P);
  if (S)
  {
    ok = ok && upload_critical_springs(parnum, sprnum, sprpart, sprpnt, sprdir, spring, spridx, dashpot, dashidx,
                                       inverse, invm, position, sprflg);
    std::vector<int> first;
    std::vector<int4> ev, bigv;
    pg_spring_events(parnum, (int)S, sprpart[0], sprpart[1], first, ev, bigv);
    ok = ok && up(d.sev_first, first.data(), P + 1) && up(d.sev, ev.data(), ev.size());
  }
  for (int k = 0; ok && k < 3; k ++) ok = grow(d.akact[k], P);
  for (int k = 0; ok && k < 6; k ++) ok = grow(d.akrot[k], P);
  ok = ok && grow(d.akmax, P) && grow(d.aemax, P) && grow(G.crit_ke, 2 * std::max<size_t>(S, 1)) &&
       grow(G.crit_h, P) && grow(G.crit_o, P) && grow(G.crit_r, P);
  if (!ok) return big;
  PgDev v = view();
  v.parnum = parnum;
  v.sprnum = (int)S;
  if (!contacts) { v.ellnum = 0; v.pell = nullptr; }
  pg_launch_critical_perparticle(v, G.st, G.crit_ke, contacts ? 1 : 0, G.crit_h, G.crit_o, G.crit_r);
  G.launches += S ? 2 : 1;
  for (int k = 0; ok && k < 3; k ++) ok = down(kact ? kact[k] : nullptr, d.akact[k], P);
  for (int k = 0; ok && k < 6; k ++) ok = down(krot ? krot[k] : nullptr, d.akrot[k], P);
  ok = ok && down(kmax, d.akmax, P) && down(emax, d.aemax, P);
  std::vector<double> hv(hcri ? 0 : P);
  double *hout = hcri ? hcri : hv.data();
  ok = ok && down(hout, G.crit_h, P) && down(ocri, G.crit_o, P) && down(rcri, G.crit_r, P);
  if (!ok || !finish("critical_perparticle")) return big;
  double hmin = big;
  for (size_t i = 0; i < P; i ++) hmin = hout[i] < hmin ? hout[i] : hmin;
  return hmin;
}

// ---------------------------------------------------------------- additions
int pg_compat_status(void)
{
  std::lock_guard<std::mutex> g(M);
  const int s = G.status;
  G.status = PG_OK;
  return s;
}

void pg_compat_exit_on_error(int on) { std::lock_guard<std::mutex> g(M); G.exit_on_error = on ? 1 : 0; }
void pg_compat_set_bits(int compat) { std::lock_guard<std::mutex> g(M); G.bits = compat; }

void pg_compat_set_skin(double skin)
{
  std::lock_guard<std::mutex> g(M);
  G.skin = skin > 0.0 ? skin : 0.0;
  G.lists = false;                            // lists of the old skin restart
}

long long pg_compat_kernel_launches(void) { std::lock_guard<std::mutex> g(M); return G.launches; }

int pg_compat_materialize(master_conpnt *master, slave_conpnt *slave, int parnum)
{
  std::lock_guard<std::mutex> g(M);
  if (!master || parnum < 0) return PG_ERR_ARGUMENT;
  for (int p = 0; p < parnum; p ++)
  {
    for (master_conpnt *q = master[p].next; q;) { master_conpnt *n = q->next; delete q; q = n; }
    master[p].next = nullptr;
    master[p].size = 0;
    if (slave)
    {
      for (slave_conpnt *q = slave[p].next; q;) { slave_conpnt *n = q->next; delete q; q = n; }
      slave[p].next = nullptr;
      slave[p].size = 0;
    }
  }
  if (!G.init || !G.lists || G.owner != (const void *)master || G.P != parnum) return 0;
  PgDev &d = G.d;
  const int E = G.E, kn = d.kn;
  const size_t n = (size_t)kn * E;
  std::vector<int> cnt(E), code(n);
  std::vector<unsigned char> flag(n);
  std::vector<double> st[3], fr[3], pt[3], nr[3], dep(n);
  bool ok = down(cnt.data(), d.ncnt, E) && down(code.data(), d.ncode, n) && down(flag.data(), d.nflag, n) &&
            down(dep.data(), d.ndep, n);
  for (int k = 0; ok && k < 3; k ++)
  {
    st[k].resize(n); fr[k].resize(n); pt[k].resize(n); nr[k].resize(n);
    ok = down(st[k].data(), d.nstate[k], n) && down(fr[k].data(), d.nfrc[k], n) && down(pt[k].data(), d.npnt[k], n) &&
         down(nr[k].data(), d.nnrm[k], n);
  }
  if (!ok || !cuda_ok(cudaStreamSynchronize(G.st), "pg_compat_materialize")) return PG_ERR_CUDA;
  int total = 0;
  for (int i = 0; i < E; i ++)
    for (int k = 0; k < cnt[i]; k ++)
    {
      const size_t idx = (size_t)k * E + i;
      if (!flag[idx]) continue;
      const int p = G.h_part[i], c = code[idx];
      master_conpnt *b = &master[p];
      while (b->size == PG_ISPC_CONBUF)
      {
        if (!b->next) { b->next = new master_conpnt(); b->next->lock = -1; }
        b = b->next;
      }
      const int s = b->size ++;
      b->master[s] = i;
      b->slave[0][s] = c >= 0 ? G.h_part[c] : G.h_triobs[-c - 1];
      b->slave[1][s] = c;
      b->color[0][s] = G.h_ellcol[i];
      b->color[1][s] = c >= 0 ? G.h_ellcol[c] : G.h_tricol[-c - 1];
      for (int a = 0; a < 3; a ++)
      {
        b->point[a][s] = pt[a][idx];
        b->normal[a][s] = nr[a][idx];
        b->force[a][s] = fr[a][idx];
        b->state[a][s] = st[a][idx];
      }
      b->depth[s] = dep[idx];
      total ++;
      const int q = b->slave[0][s];
      if (slave && q >= 0 && q < parnum)
      {
        slave_conpnt *r = &slave[q];
        while (r->size == PG_ISPC_CONBUF)
        {
          if (!r->next) { r->next = new slave_conpnt(); r->next->lock = -1; }
          r = r->next;
        }
        const int u = r->size ++;
        r->master[0][u] = p;
        r->master[1][u] = i;
        for (int a = 0; a < 3; a ++) { r->point[a][u] = pt[a][idx]; r->force[a][u] = -fr[a][idx]; }
      }
    }
  return total;
}

} // extern "C"
} // namespace ispc
