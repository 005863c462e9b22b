// pg_session.cu -- device-resident session: the C ABI of include/parmec_gb300.h.
//
// A session owns one scene in HBM.  pg_session_run enqueues, for every step,
// the rebuild kernels (they return at once unless a rebuild is due) and the
// step kernels on the session stream; host inputs of each step come from a
// device copy of the per-step table.  Nothing falls back to the CPU.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <cmath>
#include "pg_state.h"
#include "pg_launch.h"
#include "pg_meshcontact.h"
#include "../../include/parmec_gb300.h"

#define PG_GRAPH_STEPS 8          // steps per replay of the multi-step graph

struct pg_session
{
  PgDev d;
  cudaStream_t stream = nullptr;
  std::vector<void *> allocs;
  int tab_cap = 0;
  long long launches = 0;
  double ext[3] = {1.0, 1.0, 1.0}, rmax = 0.0, rmin = 0.0;
  std::vector<double> sorg_h;              // [3][nscene] grid origins
  std::vector<int> stbeg_h, stend_h;
  size_t ncells = 0;
  int prs_stride = 3, obs_stride = 3;
  std::vector<int> h_pell;
  std::vector<int> h_part;                 // sphere -> particle map the device's eorder was built from
  // per kernel group timing with CUDA events on the session stream
  int profile = 0;
  cudaEvent_t ev[8] = {};
  double group_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  long long group_launches[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  std::vector<cudaEvent_t> ring;
  // one captured step (re-captured when kernel arguments change)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  double graph_step = 0.0;
  int graph_adapt = 0;                     // the captured step is the adaptive one
  int use_graph = 1;
  // PG_GRAPH_STEPS copies of the same step in one graph (fewer graph
  // launches for long runs); dropped with the one-step graph
  cudaGraph_t graphn = nullptr;
  cudaGraphExec_t graphn_exec = nullptr;
  // adaptive stepping: device step pair, per-step records and the minimum
  // (PgDev.hs points at hs_buf only while an adaptive run is enqueued)
  double *hs_buf = nullptr;
  int adapt_ready = 0, hrec_cap = 0, sbig_ad_cap = 0;
  // mesh-mesh contact (pg_meshcontact.cu); steps then run without graphs
  PgTT tt;
  // a pool's live extents (pg_session_set_live): the steps cover particles,
  // spheres and triangles below them; 0: the whole arrays
  int plive = 0, elive = 0, tlive = 0;
  // CRITICAL: per-spring slope and damping, and the per-item outputs
  double *crit_ke = nullptr, *crit_h = nullptr, *crit_o = nullptr, *crit_r = nullptr;
  int exc_any = 0;                         // some scene has a device excitation
  // partial downloads: device scratch for indices, column table and rows
  int *g_idx = nullptr; const double **g_cols = nullptr; double *g_out = nullptr;
  size_t g_idx_cap = 0, g_cols_cap = 0, g_out_cap = 0;
  // persistent fused step (mixed form): launch shape, autotuner state and
  // the captured graph of one chunk of fstep_chunk steps
  int fused = 0, tune = 0, tuned = 0, warmed = 0;
  PgFusedCfg fcfg = {-1, 0, 0};
  std::vector<PgFusedCfg> cands;
  std::vector<double> cand_ms;
  int cand_next = 0, cand_round = 0;
  cudaGraph_t fgraph = nullptr;
  cudaGraphExec_t fgraph_exec = nullptr;
  double fgraph_step = 0.0;
  int fgraph_chunk = 0, fgraph_ok = 1;
  long long fused_launches = 0;
};

// spring force flush events per particle (CSR 'first' over particles), in
// the order one springs_task applies them (forces.ispc:1207-1412): springs
// sorted by (part0, part1) flush a run of equal part0 with += and a run of
// equal part1 with -=; 'w' marks the first run of its kind, which assigns
void pg_spring_events(int P, int S, const int *sj, const int *sk, std::vector<int> &first, std::vector<int4> &evv,
                      std::vector<int4> &big)
{
  struct Ev { int part; long long pos; int4 v; };
  std::vector<Ev> ev;
  int j0 = -1, k0 = -1, jb = 0, kb = 0;
  bool firstj = true, firstk = true;
  for (int i = 0; i < S; i ++)
  {
    int j = sj[i], k = sk[i];
    if (j0 != j && j0 >= 0)
    {
      ev.push_back({j0, 2LL*i, make_int4(0, jb, i, firstj ? 1 : 0)});
      firstj = false;
      jb = i;
    }
    if (j0 < 0) jb = i;
    if (k >= 0)
    {
      if (k0 != k && k0 >= 0)
      {
        ev.push_back({k0, 2LL*i + 1, make_int4(1, kb, i, firstk ? 1 : 0)});
        firstk = false;
        kb = i;
      }
      if (k0 < 0) kb = i;
      k0 = k;
    }
    j0 = j;
  }
  if (j0 >= 0) ev.push_back({j0, 2LL*S, make_int4(0, jb, S, firstj ? 1 : 0)});
  if (k0 >= 0) ev.push_back({k0, 2LL*S + 1, make_int4(1, kb, S, firstk ? 1 : 0)});
  std::stable_sort(ev.begin(), ev.end(), [](const Ev &a, const Ev &b) {
    return a.part != b.part ? a.part < b.part : a.pos < b.pos; });
  first.assign(P + 1, 0);
  evv.assign(std::max<size_t>(1, ev.size()), make_int4(0, 0, 0, 0));
  big.clear();
  for (size_t q = 0; q < ev.size(); q ++)
  {
    first[ev[q].part + 1] ++;
    evv[q] = ev[q].v;
    // a long run is summed by its own block beforehand (k_spring_runs); its
    // index + 1 sits above the run type in .x
    if (ev[q].v.z - ev[q].v.y > PG_SPRING_RUN_LONG)
    {
      big.push_back(ev[q].v);
      evv[q].x |= (int)big.size() << 1;
    }
  }
  for (int p = 0; p < P; p ++) first[p+1] += first[p];
}

namespace {

#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { \
  std::fprintf(stderr, "parmec_gb300: %s failed: %s (%s:%d)\n", #x, cudaGetErrorString(e_), __FILE__, __LINE__); \
  return PG_ERR_CUDA; } } while (0)

template <typename T>
int dalloc(pg_session *s, T **p, size_t n)
{
  if (n == 0) n = 1;
  void *q = nullptr;
  CK(cudaMalloc(&q, n * sizeof(T)));
  CK(cudaMemsetAsync(q, 0, n * sizeof(T), s->stream));
  s->allocs.push_back(q);
  *p = (T *)q;
  return PG_OK;
}

template <typename T>
int h2d(pg_session *s, T *dst, const T *src, size_t n)
{
  if (n == 0 || src == nullptr) return PG_OK;
  CK(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyHostToDevice, s->stream));
  return PG_OK;
}

template <typename T>
int d2h(pg_session *s, T *dst, const T *src, size_t n)
{
  if (n == 0 || dst == nullptr) return PG_OK;
  CK(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToHost, s->stream));
  return PG_OK;
}

#define TRY(x) do { int r_ = (x); if (r_ != PG_OK) return r_; } while (0)

void drop_graph(pg_session *s);

int table_len(const int *idx, int n) { return n > 0 && idx ? idx[n] : 0; }

// allocate every device array for the counts of 'sc'
int allocate(pg_session *s, const pg_scene *sc)
{
  PgDev &d = s->d;
  const size_t P = sc->parnum, E = sc->ellnum, T = sc->trinum, O = sc->obsnum;
  const size_t N = sc->nodnum, F = sc->facnum, S = sc->sprnum;
  for (int k = 0; k < 6; k ++) TRY(dalloc(s, &d.angular[k], P));
  for (int k = 0; k < 3; k ++) TRY(dalloc(s, &d.linear[k], P));
  for (int k = 0; k < 9; k ++) TRY(dalloc(s, &d.rotation[k], P));
  for (int k = 0; k < 6; k ++) TRY(dalloc(s, &d.position[k], P));
  for (int k = 0; k < 9; k ++) TRY(dalloc(s, &d.inertia[k], P));
  for (int k = 0; k < 9; k ++) TRY(dalloc(s, &d.inverse[k], P));
  TRY(dalloc(s, &d.mass, P));
  TRY(dalloc(s, &d.invm, P));
  for (int k = 0; k < 3; k ++) { TRY(dalloc(s, &d.force[k], P)); TRY(dalloc(s, &d.torque[k], P)); }
  TRY(dalloc(s, &d.flags, P));
  TRY(dalloc(s, &d.parmat, P));
  TRY(dalloc(s, &d.pell, P));
  TRY(dalloc(s, &d.piso, P));
  for (int k = 0; k < 6; k ++) TRY(dalloc(s, &d.center[k], E));
  for (int k = 0; k < 3; k ++) TRY(dalloc(s, &d.radii[k], E));
  TRY(dalloc(s, &d.ellcol, E));
  TRY(dalloc(s, &d.part, E));
  for (int k = 0; k < 9; k ++) TRY(dalloc(s, &d.tri[k], T));
  TRY(dalloc(s, &d.tricol, T));
  TRY(dalloc(s, &d.triobs, T));
  TRY(dalloc(s, &d.triown, T));
  TRY(dalloc(s, &d.trirng, 2*O));
  TRY(dalloc(s, &d.obspnt, 3*O));
  TRY(dalloc(s, &d.obsang, 3*O));
  TRY(dalloc(s, &d.obslin, 3*O));
  TRY(dalloc(s, &d.pairs, 2*(size_t)sc->pairnum));
  TRY(dalloc(s, &d.ikind, (size_t)sc->pairnum));
  for (int k = 0; k < 7; k ++) TRY(dalloc(s, &d.iparam[k], (size_t)sc->pairnum));
  for (int k = 0; k < 6; k ++) TRY(dalloc(s, &d.nodes[k], N));
  TRY(dalloc(s, &d.nodpart, N));
  for (int k = 0; k < 3; k ++) TRY(dalloc(s, &d.facnod[k], F));
  TRY(dalloc(s, &d.factri, F));
  // springs
  TRY(dalloc(s, &d.sprtype, S));
  TRY(dalloc(s, &d.unspring, S));
  for (int k = 0; k < 2; k ++) TRY(dalloc(s, &d.sprpart[k], S));
  for (int k = 0; k < 12; k ++) TRY(dalloc(s, &d.sprpnt[k], S));
  const size_t ns = table_len(sc->spridx, sc->sprnum), nd = table_len(sc->dashidx, sc->sprnum);
  const size_t nu = table_len(sc->unidx, sc->sprnum);
  for (int k = 0; k < 2; k ++)
  {
    TRY(dalloc(s, &d.spring[k], ns));
    TRY(dalloc(s, &d.dashpot[k], nd));
    TRY(dalloc(s, &d.unload[k], nu));
    TRY(dalloc(s, &d.yield[k], S));
  }
  TRY(dalloc(s, &d.spridx, S + 1));
  TRY(dalloc(s, &d.dashidx, S + 1));
  TRY(dalloc(s, &d.unidx, S + 1));
  for (int k = 0; k < 6; k ++) TRY(dalloc(s, &d.sprdir[k], S));
  TRY(dalloc(s, &d.sprflg, S));
  TRY(dalloc(s, &d.sproffset, S));
  TRY(dalloc(s, &d.sprfric, S));
  TRY(dalloc(s, &d.sprkskn, S));
  for (int k = 0; k < 3; k ++)
  {
    TRY(dalloc(s, &d.sprsdsp[k], S));
    TRY(dalloc(s, &d.stroke[k], S));
    TRY(dalloc(s, &d.sprfrc[k], S));
  }
  TRY(dalloc(s, &d.stroke0, S));
  for (int k = 0; k < 9; k ++) TRY(dalloc(s, &d.spr_out[k], S));
  // scenes
  const size_t NS = d.nscene;
  TRY(dalloc(s, &d.pscene, P));
  TRY(dalloc(s, &d.escene, E));
  TRY(dalloc(s, &d.tscene, T));
  TRY(dalloc(s, &d.oscene, O));
  TRY(dalloc(s, &d.sactive, NS));
  TRY(dalloc(s, &d.stbeg, NS));
  TRY(dalloc(s, &d.stend, NS));
  for (int k = 0; k < 3; k ++) TRY(dalloc(s, &d.sorg[k], NS));
  TRY(dalloc(s, &d.sexc_on, NS));
  TRY(dalloc(s, &d.sexc, (size_t)PG_EXC_LEN * NS));
  TRY(dalloc(s, &d.sgrav, 3 * NS));
  TRY(dalloc(s, &d.sstart, NS));
  TRY(dalloc(s, &d.gstep, 1));
  TRY(dalloc(s, &d.gbar, 4));
  return PG_OK;
}

// arrays that depend on counts only and never change during a session
int upload_static(pg_session *s, const pg_scene *sc)
{
  PgDev &d = s->d;
  const int P = sc->parnum, E = sc->ellnum, T = sc->trinum, O = sc->obsnum;
  (void)E; (void)T; (void)O;
  // prescriptions per particle, in input order
  {
    std::vector<int> first(P + 1, 0), list(std::max(1, sc->prsnum));
    for (int q = 0; q < sc->prsnum; q ++) first[sc->prspart[q] + 1] ++;
    for (int p = 0; p < P; p ++) first[p+1] += first[p];
    std::vector<int> fill(first.begin(), first.end() - 1);
    for (int q = 0; q < sc->prsnum; q ++) list[fill[sc->prspart[q]] ++] = q;
    TRY(dalloc(s, &d.prs_first, P + 1));
    TRY(dalloc(s, &d.prs_list, list.size()));
    TRY(dalloc(s, &d.prslin, std::max(1, sc->prsnum)));
    TRY(dalloc(s, &d.prsang, std::max(1, sc->prsnum)));
    TRY(dalloc(s, &d.linkind, std::max(1, sc->prsnum)));
    TRY(dalloc(s, &d.angkind, std::max(1, sc->prsnum)));
    TRY(h2d(s, d.prs_first, first.data(), P + 1));
    TRY(h2d(s, d.prs_list, list.data(), list.size()));
    TRY(h2d(s, d.prslin, sc->prslin, sc->prsnum));
    TRY(h2d(s, d.prsang, sc->prsang, sc->prsnum));
    TRY(h2d(s, d.linkind, sc->linkind, sc->prsnum));
    TRY(h2d(s, d.angkind, sc->angkind, sc->prsnum));
  }
  // restraints per particle, in input order
  {
    const int R = std::max(sc->rstnum, 0);
    std::vector<int> first(P + 1, 0), list(std::max(1, R));
    for (int q = 0; q < R; q ++) first[sc->rstpart[q] + 1] ++;
    for (int p = 0; p < P; p ++) first[p+1] += first[p];
    std::vector<int> fill(first.begin(), first.end() - 1);
    for (int q = 0; q < R; q ++) list[fill[sc->rstpart[q]] ++] = q;
    d.rstnum = R;
    TRY(dalloc(s, &d.rst_first, P + 1));
    TRY(dalloc(s, &d.rst_list, list.size()));
    TRY(h2d(s, d.rst_first, first.data(), P + 1));
    TRY(h2d(s, d.rst_list, list.data(), list.size()));
    for (int k = 0; k < 9; k ++)
    {
      TRY(dalloc(s, &d.rstlin[k], std::max(1, R)));
      TRY(dalloc(s, &d.rstang[k], std::max(1, R)));
      TRY(h2d(s, d.rstlin[k], sc->rstlin[k], R));
      TRY(h2d(s, d.rstang[k], sc->rstang[k], R));
    }
  }
  // torsion springs: tables, directions and their flush events
  {
    const int Q = std::max(sc->trqsprnum, 0);
    d.trqsprnum = Q;
    const size_t n = std::max(1, Q);
    for (int a = 0; a < 2; a ++) { TRY(dalloc(s, &d.trqsprpart[a], n)); TRY(h2d(s, d.trqsprpart[a], sc->trqsprpart[a], Q)); }
    for (int c = 0; c < 3; c ++)
    {
      TRY(dalloc(s, &d.trqzdir0[c], n)); TRY(h2d(s, d.trqzdir0[c], sc->trqzdir0[c], Q));
      TRY(dalloc(s, &d.trqxdir0[c], n)); TRY(h2d(s, d.trqxdir0[c], sc->trqxdir0[c], Q));
      TRY(dalloc(s, &d.trqzdir1[c], n)); TRY(dalloc(s, &d.trqxdir1[c], n));
      TRY(dalloc(s, &d.trqrpy[c], n)); TRY(dalloc(s, &d.trqrpytot[c], n)); TRY(dalloc(s, &d.trqrpyspr[c], n));
      TRY(dalloc(s, &d.tq_out[c], n));
    }
    for (int o = 0; o < 3; o ++)
    {
      const size_t nk = Q ? (size_t)sc->krpyidx[o][Q] : 0, nd = Q ? (size_t)sc->drpyidx[o][Q] : 0;
      TRY(dalloc(s, &d.krpyidx[o], n + 1)); TRY(h2d(s, d.krpyidx[o], sc->krpyidx[o], Q ? Q + 1 : 0));
      TRY(dalloc(s, &d.drpyidx[o], n + 1)); TRY(h2d(s, d.drpyidx[o], sc->drpyidx[o], Q ? Q + 1 : 0));
      for (int c = 0; c < 2; c ++)
      {
        TRY(dalloc(s, &d.krpy[o][c], std::max<size_t>(1, nk))); TRY(h2d(s, d.krpy[o][c], sc->krpy[o][c], nk));
        TRY(dalloc(s, &d.drpy[o][c], std::max<size_t>(1, nd))); TRY(h2d(s, d.drpy[o][c], sc->drpy[o][c], nd));
      }
    }
    TRY(dalloc(s, &d.trqcone, n)); TRY(h2d(s, d.trqcone, sc->trqcone, Q));
    std::vector<int> first;
    std::vector<int4> evv, big;
    pg_spring_events(P, Q, Q ? sc->trqsprpart[0] : nullptr, Q ? sc->trqsprpart[1] : nullptr, first, evv, big);
    for (auto &e : evv) e.x &= 1;               // torsion runs are summed whole
    TRY(dalloc(s, &d.tev_first, P + 1));
    TRY(dalloc(s, &d.tev, evv.size()));
    TRY(h2d(s, d.tev_first, first.data(), P + 1));
    TRY(h2d(s, d.tev, evv.data(), evv.size()));
    CK(cudaStreamSynchronize(s->stream));
  }
  // prescribed body forces: record storage (values and the particle map come with each upload)
  {
    d.pbfnum = std::max(sc->pbfnum, 0);
    const size_t n = std::max(1, d.pbfnum);
    TRY(dalloc(s, &d.pbf_slot, (size_t)std::max(P, 1)));
    for (int c = 0; c < 6; c ++) { TRY(dalloc(s, &d.pbfout[c], n)); TRY(dalloc(s, &d.pbfin[c], n)); }
  }
  // spring failure rules, spring ids mapped to sorted positions
  {
    const int U = std::max(sc->unsprnum, 0);
    d.unsprnum = U;
    auto mapped = [&](const int *ids, const int *idx, int **dl, int **di) -> int {
      const int n = U ? idx[U] : 0;
      std::vector<int> pos(std::max(1, n)), ix(U + 1, 0);
      for (int j = 0; j < n; j ++)
      {
        const int id = ids[j];
        if (id < 0 || id >= sc->sprnum) return PG_ERR_ARGUMENT;
        pos[j] = sc->sprmap ? sc->sprmap[id] : id;
      }
      for (int i = 0; i <= U; i ++) ix[i] = U ? idx[i] : 0;
      TRY(dalloc(s, dl, pos.size()));
      TRY(dalloc(s, di, ix.size()));
      TRY(h2d(s, *dl, pos.data(), pos.size()));
      TRY(h2d(s, *di, ix.data(), ix.size()));
      CK(cudaStreamSynchronize(s->stream));
      return PG_OK;
    };
    TRY(mapped(sc->tsprings, sc->tspridx, &d.u_t, &d.u_tidx));
    TRY(mapped(sc->msprings, sc->mspridx, &d.u_m, &d.u_midx));
    TRY(mapped(sc->activate, sc->actidx, &d.u_a, &d.u_aidx));
    const size_t n = std::max(1, U);
    for (int k = 0; k < 2; k ++) { TRY(dalloc(s, &d.unlim[k], n)); TRY(h2d(s, d.unlim[k], sc->unlim[k], U)); }
    TRY(dalloc(s, &d.unent, n)); TRY(h2d(s, d.unent, sc->unent, U));
    TRY(dalloc(s, &d.unop, n)); TRY(h2d(s, d.unop, sc->unop, U));
    TRY(dalloc(s, &d.unabs, n)); TRY(h2d(s, d.unabs, sc->unabs, U));
    TRY(dalloc(s, &d.unsteps, n)); TRY(h2d(s, d.unsteps, sc->nsteps, U));
    TRY(dalloc(s, &d.nfreq, n)); TRY(h2d(s, d.nfreq, sc->nfreq, U));
    TRY(dalloc(s, &d.unaction, n)); TRY(h2d(s, d.unaction, sc->unaction, U));
    TRY(dalloc(s, &d.ustep, 1));
  }
  // spring flush events: the single-task springs_task order (forces.ispc:1207-1412)
  {
    std::vector<int> first;
    std::vector<int4> evv, big;
    pg_spring_events(P, sc->sprnum, sc->sprpart[0], sc->sprpart[1], first, evv, big);
    TRY(dalloc(s, &d.sev_first, P + 1));
    TRY(dalloc(s, &d.sev, evv.size()));
    TRY(h2d(s, d.sev_first, first.data(), P + 1));
    TRY(h2d(s, d.sev, evv.data(), evv.size()));
    d.nbig = (int)big.size();
    TRY(dalloc(s, &d.sbig, std::max<size_t>(1, big.size())));
    TRY(dalloc(s, &d.sbig_sum, 6 * std::max<size_t>(1, big.size())));
    TRY(dalloc(s, &d.sbig_grp, 32 * 12 * std::max<size_t>(1, big.size())));
    TRY(h2d(s, d.sbig, big.data(), big.size()));
    CK(cudaStreamSynchronize(s->stream));
  }
  return PG_OK;
}

struct Ranges { size_t p0, p1, e0, e1, t0, t1, o0, o1; };

Ranges full_ranges(const PgDev &d)
{
  return {0, (size_t)d.parnum, 0, (size_t)d.ellnum, 0, (size_t)d.trinum, 0, (size_t)d.obsnum};
}

template <typename T>
int h2dr(pg_session *s, T *dst, const T *src, size_t b, size_t e, size_t w = 1)
{
  if (e <= b || !src) return PG_OK;
  return h2d(s, dst + w * b, src + w * b, w * (e - b));
}

template <typename T>
int d2hr(pg_session *s, T *dst, const T *src, size_t b, size_t e, size_t w = 1)
{
  if (e <= b || !dst) return PG_OK;
  return d2h(s, dst + w * b, src + w * b, w * (e - b));
}

// triangle ranges of every scene from the host's triangle -> scene map
int scene_triangle_ranges(pg_session *s, const pg_scene *sc)
{
  PgDev &d = s->d;
  s->stbeg_h.assign(d.nscene, 0);
  s->stend_h.assign(d.nscene, 0);
  std::vector<int> seen(d.nscene, 0);
  for (int t = 0; t < d.trinum; t ++)
  {
    int k = (sc->nscene && sc->tscene) ? sc->tscene[t] : 0;
    if (k < 0) continue;                                   // a triangle of no scene
    if (k >= d.nscene) return PG_ERR_ARGUMENT;
    if (!seen[k]) { s->stbeg_h[k] = t; seen[k] = 1; }
    else if (s->stend_h[k] != t) return PG_ERR_ARGUMENT;   // a scene's triangles must be contiguous
    s->stend_h[k] = t + 1;
  }
  TRY(h2d(s, d.stbeg, s->stbeg_h.data(), d.nscene));
  TRY(h2d(s, d.stend, s->stend_h.data(), d.nscene));
  return PG_OK;
}

// copy the given ranges of every per-particle, per-sphere, per-triangle and
// per-obstacle array; 'global' also copies pairs, springs, meshes and curves
int upload_ranges(pg_session *s, const pg_scene *sc, Ranges r, bool global, bool restart_lists)
{
  PgDev &d = s->d;
  const size_t p0 = r.p0, p1 = r.p1, e0 = r.e0, e1 = r.e1, t0 = r.t0, t1 = r.t1, o0 = r.o0, o1 = r.o1;
  for (int k = 0; k < 6; k ++) TRY(h2dr(s, d.angular[k], sc->angular[k], p0, p1));
  for (int k = 0; k < 3; k ++) TRY(h2dr(s, d.linear[k], sc->linear[k], p0, p1));
  for (int k = 0; k < 9; k ++) TRY(h2dr(s, d.rotation[k], sc->rotation[k], p0, p1));
  for (int k = 0; k < 6; k ++) TRY(h2dr(s, d.position[k], sc->position[k], p0, p1));
  for (int k = 0; k < 9; k ++) TRY(h2dr(s, d.inertia[k], sc->inertia[k], p0, p1));
  for (int k = 0; k < 9; k ++) TRY(h2dr(s, d.inverse[k], sc->inverse[k], p0, p1));
  TRY(h2dr(s, d.mass, sc->mass, p0, p1));
  TRY(h2dr(s, d.invm, sc->invm, p0, p1));
  for (int k = 0; k < 3; k ++) { TRY(h2dr(s, d.force[k], sc->force[k], p0, p1)); TRY(h2dr(s, d.torque[k], sc->torque[k], p0, p1)); }
  TRY(h2dr(s, d.flags, sc->flags, p0, p1));
  TRY(h2dr(s, d.parmat, sc->parmat, p0, p1));
  for (int k = 0; k < 6; k ++) TRY(h2dr(s, d.center[k], sc->center[k], e0, e1));
  for (int k = 0; k < 3; k ++) TRY(h2dr(s, d.radii[k], sc->radii[k], e0, e1));
  TRY(h2dr(s, d.ellcol, sc->ellcol, e0, e1));
  TRY(h2dr(s, d.part, sc->part, e0, e1));
  for (int v = 0; v < 3; v ++)
    for (int c = 0; c < 3; c ++) TRY(h2dr(s, d.tri[3*v+c], sc->tri[v][c], t0, t1));
  TRY(h2dr(s, d.tricol, sc->tricol, t0, t1));
  TRY(h2dr(s, d.triobs, sc->triobs, t0, t1));
  TRY(h2dr(s, d.trirng, sc->trirng, o0, o1, 2));
  TRY(h2dr(s, d.obspnt, sc->obspnt, o0, o1, 3));
  TRY(h2dr(s, d.obsang, sc->obsang, o0, o1, 3));
  TRY(h2dr(s, d.obslin, sc->obslin, o0, o1, 3));

  // particle -> sphere for the particles of the range
  {
    std::vector<int> pell(p1 - p0, -1);
    for (size_t e = e0; e < e1; e ++)
    {
      int p = sc->part[e];
      if (p < 0 || p >= d.parnum) return PG_ERR_ARGUMENT;
      if (!(sc->radii[1][e] < 0.0)) return PG_ERR_UNSUPPORTED;   // ellipsoids: assert(0) in the reference
      if ((size_t)p >= p0 && (size_t)p < p1)
      {
        if (pell[p - p0] >= 0) return PG_ERR_UNSUPPORTED;       // more than one sphere per particle
        pell[p - p0] = (int)e;
      }
    }
    if (s->h_pell.size() != (size_t)d.parnum) s->h_pell.assign(d.parnum, -1);
    for (size_t p = p0; p < p1; p ++) s->h_pell[p] = pell[p - p0];
    TRY(h2dr(s, d.pell, s->h_pell.data(), p0, p1));
  }
  // spheres in particle order (stable): the order of the slave-list entries.
  // It depends on the sphere -> particle map alone, so an upload that leaves
  // the map of its range as it was (the next DEM call of the same model, a
  // pooled scene loaded into its own ranges) keeps the order already on the
  // device.
  if (d.ellnum)
  {
    bool same = s->h_part.size() == (size_t)d.ellnum;
    for (size_t e = e0; same && e < e1; e ++) same = s->h_part[e] == sc->part[e];
    if (!same)
    {
      s->h_part.assign(sc->part, sc->part + d.ellnum);
      std::vector<int> ord(d.ellnum);
      for (int e = 0; e < d.ellnum; e ++) ord[e] = e;
      std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return s->h_part[a] < s->h_part[b]; });
      TRY(h2d(s, d.eorder, ord.data(), ord.size()));
      CK(cudaStreamSynchronize(s->stream));         // ord is a local
    }
  }
  // triangle -> moving obstacle for the triangles of the range
  {
    std::vector<int> own(d.trinum, -1);
    for (int o = 0; o < d.obsnum; o ++)
      for (int t = sc->trirng[2*o]; t < sc->trirng[2*o+1]; t ++)
        if (t >= 0 && t < d.trinum) own[t] = o;
    TRY(h2dr(s, d.triown, own.data(), t0, t1));
  }
  // scenes (host vectors hold the ranges only)
  {
    std::vector<int> ps(p1 - p0, 0), es(e1 - e0, 0), ts(t1 - t0, 0), os(o1 - o0, 0);
    const bool many = sc->nscene > 0;
    for (size_t p = p0; p < p1; p ++) ps[p - p0] = many ? sc->pscene[p] : 0;
    for (size_t e = e0; e < e1; e ++) es[e - e0] = many ? sc->pscene[sc->part[e]] : 0;   // -1: no scene
    for (size_t t = t0; t < t1; t ++) ts[t - t0] = many ? sc->tscene[t] : 0;
    for (size_t o = o0; o < o1; o ++) os[o - o0] = many ? sc->oscene[o] : 0;
    TRY(h2d(s, d.pscene + p0, ps.data(), ps.size()));
    TRY(h2d(s, d.escene + e0, es.data(), es.size()));
    TRY(h2d(s, d.tscene + t0, ts.data(), ts.size()));
    TRY(h2d(s, d.oscene + o0, os.data(), os.size()));
    TRY(scene_triangle_ranges(s, sc));
    CK(cudaStreamSynchronize(s->stream));           // the vectors are locals
  }
  // a newly loaded scene's spheres start with empty candidate lists; a
  // re-upload of the same scene keeps its contacts and their state
  if (restart_lists && e1 > e0) CK(cudaMemsetAsync(d.ncnt + e0, 0, (e1 - e0) * sizeof(int), s->stream));

  if (global)
  {
    const size_t N = sc->nodnum, F = sc->facnum, S = sc->sprnum;
    TRY(h2d(s, d.pairs, sc->pairs, 2*(size_t)sc->pairnum));
    TRY(h2d(s, d.ikind, sc->ikind, (size_t)sc->pairnum));
    for (int k = 0; k < 7; k ++) TRY(h2d(s, d.iparam[k], sc->iparam[k], (size_t)sc->pairnum));
    if (d.form == PG_FORM_MIXED && sc->pairnum > 0)
    {
      std::vector<float> f((size_t)sc->pairnum);
      for (int k = 0; k < 7; k ++)
      {
        for (int q = 0; q < sc->pairnum; q ++) f[q] = (float)sc->iparam[k][q];
        TRY(h2d(s, d.iparam_f[k], f.data(), f.size()));
        CK(cudaStreamSynchronize(s->stream));       // f is reused
      }
    }
    for (int k = 0; k < 6; k ++) TRY(h2d(s, d.nodes[k], sc->nodes[k], N));
    TRY(h2d(s, d.nodpart, sc->nodpart, N));
    for (int k = 0; k < 3; k ++) TRY(h2d(s, d.facnod[k], sc->facnod[k], F));
    TRY(h2d(s, d.factri, sc->factri, F));
    TRY(h2d(s, d.sprtype, sc->sprtype, S));
    TRY(h2d(s, d.unspring, sc->unspring, S));
    for (int k = 0; k < 2; k ++) TRY(h2d(s, d.sprpart[k], sc->sprpart[k], S));
    for (int a = 0; a < 2; a ++)
      for (int k = 0; k < 6; k ++) TRY(h2d(s, d.sprpnt[6*a+k], sc->sprpnt[a][k], S));
    const size_t ns = table_len(sc->spridx, sc->sprnum), nd = table_len(sc->dashidx, sc->sprnum);
    const size_t nu = table_len(sc->unidx, sc->sprnum);
    for (int k = 0; k < 2; k ++)
    {
      TRY(h2d(s, d.spring[k], sc->spring[k], ns));
      TRY(h2d(s, d.dashpot[k], sc->dashpot[k], nd));
      TRY(h2d(s, d.unload[k], sc->unload[k], nu));
      TRY(h2d(s, d.yield[k], sc->yield[k], S));
    }
    if (S)
    {
      TRY(h2d(s, d.spridx, sc->spridx, S + 1));
      TRY(h2d(s, d.dashidx, sc->dashidx, S + 1));
      TRY(h2d(s, d.unidx, sc->unidx, S + 1));
    }
    for (int k = 0; k < 6; k ++) TRY(h2d(s, d.sprdir[k], sc->sprdir[k], S));
    TRY(h2d(s, d.sprflg, sc->sprflg, S));
    TRY(h2d(s, d.sproffset, sc->sproffset, S));
    TRY(h2d(s, d.sprfric, sc->sprfric, S));
    TRY(h2d(s, d.sprkskn, sc->sprkskn, S));
    for (int k = 0; k < 3; k ++)
    {
      TRY(h2d(s, d.sprsdsp[k], sc->sprsdsp[k], S));
      TRY(h2d(s, d.stroke[k], sc->stroke[k], S));
      TRY(h2d(s, d.sprfrc[k], sc->sprfrc[k], S));
    }
    TRY(h2d(s, d.stroke0, sc->stroke0, S));
    // lookup curves used as stroke offsets (sproffset) and as UNSPRING unload
    // curves (unaction >= 0)
    int nlc = 0;
    if (sc->sproffset)
      for (size_t i = 0; i < S; i ++) nlc = std::max(nlc, sc->sproffset[i] + 1);
    if (sc->unaction)
      for (int i = 0; i < sc->unsprnum; i ++) nlc = std::max(nlc, sc->unaction[i] + 1);
    size_t nl = (nlc > 0 && sc->lcidx) ? (size_t)sc->lcidx[nlc] : 0;
    if (!d.lcidx)
    {
      TRY(dalloc(s, &d.lcidx, nlc + 1));
      for (int k = 0; k < 2; k ++) TRY(dalloc(s, &d.lcurve[k], nl));
    }
    if (nlc > 0)
    {
      TRY(h2d(s, d.lcidx, sc->lcidx, nlc + 1));
      for (int k = 0; k < 2; k ++) TRY(h2d(s, d.lcurve[k], sc->lcurve[k], nl));
    }
    std::vector<int> act(d.nscene, 1);
    if (sc->nscene && sc->sactive) for (int k = 0; k < d.nscene; k ++) act[k] = sc->sactive[k] ? 1 : 0;
    TRY(h2d(s, d.sactive, act.data(), d.nscene));
  }
  if (d.form == PG_FORM_MIXED) pg_launch_mx_from64(d, s->stream, (int)p0, (int)p1, (int)e0, (int)e1);
  else pg_launch_iso_flags(d, s->stream, (int)p0, (int)p1);
  int one = 1;
  TRY(h2d(s, d.rebuild, &one, 1));
  return PG_OK;
}

// torsion spring state (directions, angles, moments)
int torsion_state(pg_session *s, const pg_scene *sc, bool up)
{
  PgDev &d = s->d;
  const size_t Q = d.trqsprnum;
  if (!Q || sc->trqsprnum != d.trqsprnum) return PG_OK;
  for (int c = 0; c < 3; c ++)
  {
    double *dv[5] = {d.trqzdir1[c], d.trqxdir1[c], d.trqrpy[c], d.trqrpytot[c], d.trqrpyspr[c]};
    double *hv[5] = {sc->trqzdir1[c], sc->trqxdir1[c], sc->trqrpy[c], sc->trqrpytot[c], sc->trqrpyspr[c]};
    for (int a = 0; a < 5; a ++)
    {
      if (up) TRY(h2d(s, dv[a], hv[a], Q));
      else TRY(d2h(s, hv[a], dv[a], Q));
    }
  }
  return PG_OK;
}

// prescribed body forces: the outer values and the particle -> record map
int body_forces_up(pg_session *s, const pg_scene *sc)
{
  PgDev &d = s->d;
  if (!d.pbfnum || sc->pbfnum != d.pbfnum) return PG_OK;
  std::vector<int> slot(d.parnum, -1);
  for (int q = 0; q < d.pbfnum; q ++)
  {
    const int p = sc->pbfpart[q];
    if (p < 0 || p >= d.parnum) return PG_ERR_ARGUMENT;
    slot[p] = q;
  }
  TRY(h2d(s, d.pbf_slot, slot.data(), slot.size()));
  for (int c = 0; c < 6; c ++) TRY(h2d(s, d.pbfout[c], sc->pbfout[c], (size_t)d.pbfnum));
  CK(cudaStreamSynchronize(s->stream));
  return PG_OK;
}

int upload_all(pg_session *s, const pg_scene *sc)
{
  TRY(upload_ranges(s, sc, full_ranges(s->d), true, false));
  TRY(body_forces_up(s, sc));
  return torsion_state(s, sc, true);
}

int download_ranges(pg_session *s, pg_scene *sc, Ranges r)
{
  PgDev &d = s->d;
  const size_t p0 = r.p0, p1 = r.p1, e0 = r.e0, e1 = r.e1, t0 = r.t0, t1 = r.t1, o0 = r.o0, o1 = r.o1;
  if (d.form == PG_FORM_MIXED) pg_launch_mx_to64(d, s->stream, (int)p0, (int)p1);
  for (int k = 0; k < 6; k ++) TRY(d2hr(s, sc->angular[k], d.angular[k], p0, p1));
  for (int k = 0; k < 3; k ++) TRY(d2hr(s, sc->linear[k], d.linear[k], p0, p1));
  for (int k = 0; k < 9; k ++) TRY(d2hr(s, sc->rotation[k], d.rotation[k], p0, p1));
  for (int k = 0; k < 6; k ++) TRY(d2hr(s, sc->position[k], d.position[k], p0, p1));
  for (int k = 0; k < 9; k ++) TRY(d2hr(s, sc->inverse[k], d.inverse[k], p0, p1));
  TRY(d2hr(s, sc->invm, d.invm, p0, p1));
  for (int k = 0; k < 3; k ++) { TRY(d2hr(s, sc->force[k], d.force[k], p0, p1)); TRY(d2hr(s, sc->torque[k], d.torque[k], p0, p1)); }
  for (int k = 0; k < 3; k ++) TRY(d2hr(s, sc->center[k], d.center[k], e0, e1));
  for (int v = 0; v < 3; v ++)
    for (int c = 0; c < 3; c ++) TRY(d2hr(s, sc->tri[v][c], d.tri[3*v+c], t0, t1));
  TRY(d2hr(s, sc->obspnt, d.obspnt, o0, o1, 3));
  TRY(d2hr(s, sc->obsang, d.obsang, o0, o1, 3));
  TRY(d2hr(s, sc->obslin, d.obslin, o0, o1, 3));
  return PG_OK;
}

int ensure_tables(pg_session *s, int n)
{
  PgDev &d = s->d;
  if (n <= s->tab_cap) return PG_OK;
  int cap = std::max(n, 2 * s->tab_cap);
  drop_graph(s);
  double **arrs[7] = {&d.t_curtime, &d.t_gravity, &d.t_damping, &d.t_prs_lin, &d.t_prs_ang, &d.t_obs_ang, &d.t_obs_lin};
  size_t widths[7] = {1, 3, 6, (size_t)s->prs_stride, (size_t)s->prs_stride, (size_t)s->obs_stride, (size_t)s->obs_stride};
  for (int k = 0; k < 7; k ++)
  {
    if (*arrs[k])
    {
      CK(cudaStreamSynchronize(s->stream));
      auto it = std::find(s->allocs.begin(), s->allocs.end(), (void *)*arrs[k]);
      if (it != s->allocs.end()) s->allocs.erase(it);
      CK(cudaFree(*arrs[k]));
      *arrs[k] = nullptr;
    }
    TRY(dalloc(s, arrs[k], (size_t)cap * widths[k]));
  }
  s->tab_cap = cap;
  return PG_OK;
}

void release(pg_session *s, void *p)
{
  if (!p) return;
  auto it = std::find(s->allocs.begin(), s->allocs.end(), p);
  if (it != s->allocs.end()) s->allocs.erase(it);
  cudaFree(p);
}

// candidate-list storage: kn slots per sphere, kr slave slots per particle;
// the per-slot FP64 arrays exist only in the FP64 form
int slot_buffers(pg_session *s)
{
  PgDev &d = s->d;
  const size_t E = d.ellnum, P = d.parnum;
  const size_t slots = (size_t)d.kn * std::max<size_t>(E, 1);
  TRY(dalloc(s, &d.ncode, slots));
  TRY(dalloc(s, &d.nflag, slots));
  if (d.form == PG_FORM_FP64)
  {
    for (int k = 0; k < 3; k ++)
    {
      TRY(dalloc(s, &d.nstate[k], slots));
      TRY(dalloc(s, &d.nfrc[k], slots));
      TRY(dalloc(s, &d.npnt[k], slots));
      TRY(dalloc(s, &d.nnrm[k], slots));
    }
    TRY(dalloc(s, &d.ndep, slots));
    TRY(dalloc(s, &d.nen, slots));
    TRY(dalloc(s, &d.cwork, slots));
    TRY(dalloc(s, &d.cwork_n, 1));
  }
  else
  {
    for (int k = 0; k < 3; k ++)
    {
      TRY(dalloc(s, &d.nstate_f[k], slots));
      TRY(dalloc(s, &d.nfrc_f[k], slots));
      TRY(dalloc(s, &d.narm_f[k], slots));
    }
  }
  // slave-list entries: at most kn per sphere
  const size_t ent = slots;
  for (int k = 0; k < 2; k ++) { TRY(dalloc(s, &d.skey[k], ent)); TRY(dalloc(s, &d.sval[k], ent)); }
  const int nb = pg_sort_blocks((int)ent);
  TRY(dalloc(s, &d.shist, 256 * (size_t)nb));
  const int sb = std::max(pg_scan_blocks(256 * nb), std::max(pg_scan_blocks((int)E + 1), pg_scan_blocks((int)P + 1)));
  TRY(dalloc(s, &d.sbs, (size_t)sb));
  d.rref = d.sval[pg_sort_passes_exact(d.sbits) & 1];        // where the entry sort leaves its result
  (void)P;
  return PG_OK;
}

void release_slot_buffers(pg_session *s)
{
  PgDev &d = s->d;
  release(s, d.ncode); release(s, d.nflag); release(s, d.ndep); release(s, d.nen);
  release(s, d.cwork); release(s, d.cwork_n);
  d.ncode = nullptr; d.nflag = nullptr; d.ndep = nullptr; d.nen = nullptr; d.rref = nullptr;
  d.cwork = nullptr; d.cwork_n = nullptr;
  for (int k = 0; k < 2; k ++) { release(s, d.skey[k]); release(s, d.sval[k]); d.skey[k] = nullptr; d.sval[k] = nullptr; }
  release(s, d.shist); release(s, d.sbs); d.shist = nullptr; d.sbs = nullptr;
  for (int k = 0; k < 3; k ++)
  {
    release(s, d.nstate[k]); release(s, d.nfrc[k]); release(s, d.npnt[k]); release(s, d.nnrm[k]);
    release(s, d.nstate_f[k]); release(s, d.nfrc_f[k]); release(s, d.narm_f[k]);
    d.nstate[k] = d.nfrc[k] = d.npnt[k] = d.nnrm[k] = nullptr;
    d.nstate_f[k] = d.nfrc_f[k] = d.narm_f[k] = nullptr;
  }
}

int contact_buffers(pg_session *s)
{
  PgDev &d = s->d;
  const size_t E = d.ellnum, P = d.parnum, T = d.trinum;
  TRY(dalloc(s, &d.ncnt, E));
  for (int k = 0; k < 3; k ++)
  {
    TRY(dalloc(s, &d.fm[k], P));
    TRY(dalloc(s, &d.tm[k], P));
    TRY(dalloc(s, &d.cref[k], E));
  }
  TRY(dalloc(s, &d.cfs, E));
  TRY(dalloc(s, &d.pfs, E));
  TRY(dalloc(s, &d.ekey, E));
  TRY(dalloc(s, &d.rcnt, P));
  TRY(dalloc(s, &d.soff, P + 1));
  TRY(dalloc(s, &d.eorder, E));
  s->h_part.clear();                              // eorder is rebuilt at the next upload
  TRY(dalloc(s, &d.eoff, E + 1));
  TRY(dalloc(s, &d.smeta, 5));
  d.sbits = pg_rebuild_entry_bits((int)P);
  for (int k = 0; k < 9; k ++) TRY(dalloc(s, &d.tref[k], T));
  TRY(dalloc(s, &d.tbox, 6 * std::max<size_t>(T, 1)));
  for (int k = 0; k < 2; k ++)
  {
    TRY(dalloc(s, &d.keys[k], E));
    TRY(dalloc(s, &d.vals[k], E));
  }
  d.nsortblocks = pg_sort_blocks((int)E);
  TRY(dalloc(s, &d.hist, 256 * (size_t)d.nsortblocks));
  return slot_buffers(s);
}

int mixed_buffers(pg_session *s)
{
  PgDev &d = s->d;
  const size_t P = d.parnum, E = d.ellnum;
  for (int k = 0; k < 3; k ++)
  {
    TRY(dalloc(s, &d.xh[k], P)); TRY(dalloc(s, &d.xl[k], P));
    TRY(dalloc(s, &d.vh[k], P)); TRY(dalloc(s, &d.vl[k], P));
    TRY(dalloc(s, &d.Om[k], P)); TRY(dalloc(s, &d.om[k], P));
    TRY(dalloc(s, &d.F_f[k], P)); TRY(dalloc(s, &d.T_f[k], P));
    TRY(dalloc(s, &d.fm_f[k], P)); TRY(dalloc(s, &d.tm_f[k], P));
  }
  for (int k = 0; k < 9; k ++)
  {
    TRY(dalloc(s, &d.Lh[k], P)); TRY(dalloc(s, &d.Ll[k], P));
    TRY(dalloc(s, &d.J_f[k], P)); TRY(dalloc(s, &d.I_f[k], P));
  }
  TRY(dalloc(s, &d.mass_f, P)); TRY(dalloc(s, &d.invm_f, P));
  TRY(dalloc(s, &d.rh, E)); TRY(dalloc(s, &d.rl, E));
  TRY(dalloc(s, &d.twork, std::max<size_t>(E, 1)));   // triangle queue of the contact passes
  TRY(dalloc(s, &d.tcnt, 2));
  TRY(dalloc(s, &d.jiso, P)); TRY(dalloc(s, &d.iiso, P));
  for (int k = 0; k < 3; k ++) TRY(dalloc(s, &d.cref_f[k], E));
  for (int k = 0; k < 7; k ++) TRY(dalloc(s, &d.iparam_f[k], (size_t)std::max(d.pairnum, 1)));
  TRY(dalloc(s, &d.sgrav_f, 3 * (size_t)std::max(d.nscene, 1)));
  TRY(dalloc(s, &d.damp_f, 6));
  return PG_OK;
}

int grid_buffers(pg_session *s)
{
  PgDev &d = s->d;
  if (pg_rebuild_sort_bits(d) > 32) return PG_ERR_ARGUMENT;   // (scene, cell) keys must fit 32 bits
  drop_graph(s);
  size_t cells = (size_t)d.nscene << (3 * d.bits);
  if (cells != s->ncells)
  {
    for (int *p : {d.cstart, d.cend})
      if (p)
      {
        auto it = std::find(s->allocs.begin(), s->allocs.end(), (void *)p);
        if (it != s->allocs.end()) s->allocs.erase(it);
        CK(cudaFree(p));
      }
    TRY(dalloc(s, &d.cstart, cells));
    TRY(dalloc(s, &d.cend, cells));
    s->ncells = cells;
  }
  else
  {
    CK(cudaMemsetAsync(d.cstart, 0, cells * sizeof(int), s->stream));
    CK(cudaMemsetAsync(d.cend, 0, cells * sizeof(int), s->stream));
  }
  if (d.keys[0]) CK(cudaMemsetAsync(d.keys[0], 0, (size_t)std::max(1, d.ellnum) * sizeof(unsigned), s->stream));
  for (int k = 0; k < 3; k ++) TRY(h2d(s, d.sorg[k], s->sorg_h.data() + (size_t)k * d.nscene, d.nscene));
  int one = 1;
  TRY(h2d(s, d.rebuild, &one, 1));
  return PG_OK;
}

// per-scene sphere bounding boxes -> common cell size and dims, per-scene origins
int grid_from_scene(pg_session *s, const pg_scene *sc)
{
  PgDev &d = s->d;
  const int NS = d.nscene;
  std::vector<double> lo(3 * NS, 1e300), hi(3 * NS, -1e300);
  s->rmax = 0.0; s->rmin = 1e300;
  for (int e = 0; e < sc->ellnum; e ++)
  {
    int k = sc->nscene ? sc->pscene[sc->part[e]] : 0;
    if (k < 0) continue;
    for (int c = 0; c < 3; c ++)
    {
      lo[3*k+c] = std::min(lo[3*k+c], sc->center[c][e]);
      hi[3*k+c] = std::max(hi[3*k+c], sc->center[c][e]);
    }
    s->rmax = std::max(s->rmax, sc->radii[0][e]);
    s->rmin = std::min(s->rmin, sc->radii[0][e]);
  }
  if (!(s->rmax > 0.0)) s->rmax = s->rmin = 1e-3;   // no sphere in any scene yet (an empty pool):
                                                    // the host sets the skin and grid before loading
  for (int c = 0; c < 3; c ++) s->ext[c] = 1e-300;
  for (int k = 0; k < NS; k ++)
    for (int c = 0; c < 3; c ++)
      if (hi[3*k+c] >= lo[3*k+c]) s->ext[c] = std::max(s->ext[c], hi[3*k+c] - lo[3*k+c]);
  pg_rebuild_grid_params(d, s->ext, s->rmax, s->rmin);
  s->sorg_h.assign(3 * (size_t)NS, 0.0);
  for (int k = 0; k < NS; k ++)
    for (int c = 0; c < 3; c ++)
      s->sorg_h[(size_t)c * NS + k] = hi[3*k+c] >= lo[3*k+c] ? lo[3*k+c] - 4.0 * d.cell : 0.0;
  return grid_buffers(s);
}

void drop_graph(pg_session *s)
{
  if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
  if (s->graph) cudaGraphDestroy(s->graph);
  s->graph_exec = nullptr;
  s->graph = nullptr;
  if (s->graphn_exec) cudaGraphExecDestroy(s->graphn_exec);
  if (s->graphn) cudaGraphDestroy(s->graphn);
  s->graphn_exec = nullptr;
  s->graphn = nullptr;
  if (s->fgraph_exec) cudaGraphExecDestroy(s->fgraph_exec);
  if (s->fgraph) cudaGraphDestroy(s->fgraph);
  s->fgraph_exec = nullptr;
  s->fgraph = nullptr;
}

// the fused kernel for 'n' steps, as a captured graph of 'chunk' steps per
// replay when capture works, else as direct cooperative launches
// kernels one fused step launches: the gated centre conversion and rebuild
// (with spheres), then the fused step kernel
PgDev live_view(const pg_session *s);

static int fused_kernels_per_step(const PgDev &d) { return d.ellnum ? 3 : 1; }

int run_fused(pg_session *s, double step, int n, int chunk)
{
  const PgDev d = live_view(s);
  if (n <= 0) return PG_OK;
  if (s->use_graph && s->fgraph_ok && n >= chunk)
  {
    if (!s->fgraph_exec || s->fgraph_step != step || s->fgraph_chunk != chunk)
    {
      if (s->fgraph_exec) cudaGraphExecDestroy(s->fgraph_exec);
      if (s->fgraph) cudaGraphDestroy(s->fgraph);
      s->fgraph_exec = nullptr;
      s->fgraph = nullptr;
      cudaError_t e = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess)
      {
        cudaError_t el = pg_launch_fused_mx(d, s->stream, step, chunk, s->fcfg);
        e = cudaStreamEndCapture(s->stream, &s->fgraph);
        if (el != cudaSuccess) e = el;
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&s->fgraph_exec, s->fgraph, 0);
      if (e != cudaSuccess)
      {
        // capture of a cooperative launch not available: launch directly
        cudaGetLastError();
        if (s->fgraph) cudaGraphDestroy(s->fgraph);
        s->fgraph = nullptr;
        s->fgraph_exec = nullptr;
        s->fgraph_ok = 0;
      }
      else
      {
        s->fgraph_step = step;
        s->fgraph_chunk = chunk;
      }
    }
    if (s->fgraph_exec)
    {
      const int reps = n / chunk;
      for (int k = 0; k < reps; k ++) CK(cudaGraphLaunch(s->fgraph_exec, s->stream));
      s->fused_launches += (long long)reps * chunk * fused_kernels_per_step(d);
      n -= reps * chunk;
    }
  }
  if (n > 0)
  {
    CK(pg_launch_fused_mx(d, s->stream, step, n, s->fcfg));
    s->fused_launches += (long long)n * fused_kernels_per_step(d);
  }
  return PG_OK;
}

// the fused path of pg_session_run: the first steps of a tuning session time
// every candidate launch shape (the results do not depend on the shape), the
// rest run with the fastest
int run_fused_steps(pg_session *s, double step, int n)
{
  int done = 0;
  if (s->tune && !s->tuned)
  {
    if (s->cands.empty())
    {
      PgFusedCfg buf[32];
      const int m = pg_fused_candidates(buf, 32);
      if (m <= 0) return PG_ERR_CUDA;
      s->cands.assign(buf, buf + m);
      s->cand_ms.assign(m, 1e30);
      s->cand_next = 0;
      s->cand_round = 0;
    }
    if (!s->warmed && done < n)
    {
      // an untimed step: the first rebuild and cold caches
      CK(pg_launch_fused_mx(live_view(s), s->stream, step, 1, s->cands[0]));
      s->fused_launches += fused_kernels_per_step(s->d);
      done += 1;
      s->warmed = 1;
    }
    const int trial = 3;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    while (!s->tuned && done + trial <= n)
    {
      const PgFusedCfg &c = s->cands[s->cand_next];
      CK(cudaEventRecord(e0, s->stream));
      CK(pg_launch_fused_mx(live_view(s), s->stream, step, trial, c));
      CK(cudaEventRecord(e1, s->stream));
      s->fused_launches += (long long)trial * fused_kernels_per_step(s->d) - 1;
      CK(cudaEventSynchronize(e1));
      float ms = 0.0f;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      s->fused_launches += 1;
      s->cand_ms[s->cand_next] = std::min(s->cand_ms[s->cand_next], (double)ms);
      done += trial;
      if (++ s->cand_next == (int)s->cands.size())
      {
        s->cand_next = 0;
        if (++ s->cand_round == 2)
        {
          int best = 0;
          for (int k = 1; k < (int)s->cands.size(); k ++) if (s->cand_ms[k] < s->cand_ms[best]) best = k;
          s->fcfg = s->cands[best];
          s->tuned = 1;
          drop_graph(s);
        }
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  if (s->fcfg.shape < 0) return PG_ERR_ARGUMENT;
  return run_fused(s, step, n - done, 16);
}

int tt_stage(pg_session *s, double step);

// the view the step kernels get: the whole arrays, or a pool's live extents
// (the slot arrays keep their stride, d.estride)
PgDev live_view(const pg_session *s)
{
  PgDev v = s->d;
  if (s->plive > 0 || s->elive > 0 || s->tlive > 0)
  {
    v.parnum = s->plive;
    v.ellnum = s->elive;
    v.trinum = s->tlive;
    v.nsortblocks = pg_sort_blocks(s->elive);
  }
  return v;
}

void enqueue_step(pg_session *s, double step)
{
  const PgDev d = live_view(s);
  if (d.form == PG_FORM_MIXED) pg_launch_mx_centres(d, s->stream);
  pg_launch_rebuild(d, s->stream);
  pg_launch_excite(d, s->stream, step);
  if (d.form == PG_FORM_MIXED)
  {
    pg_launch_contacts_mx(d, s->stream, step);
    pg_launch_integrate_mx(d, s->stream, step);
    pg_launch_obstacles_tail(d, s->stream, step);
    return;
  }
  pg_launch_contacts(d, s->stream, step);
  pg_launch_springs(d, s->stream, step);
  pg_launch_spring_runs(d, s->stream);
  pg_launch_torsion(d, s->stream, step);
  pg_launch_unspring(d, s->stream);
  if (d.tt_on) tt_stage(s, step);
  pg_launch_integrate(d, s->stream, step);
  pg_launch_mesh(d, s->stream);
  pg_launch_obstacles_tail(d, s->stream, step);
}

// the mesh-contact stage of one step: pairs, forces and per-particle sums;
// it reads the pair count back (one host wait per step), so steps with mesh
// contact are not captured in graphs
int tt_stage(pg_session *s, double step)
{
  PgDev &d = s->d;
  PgTT &g = s->tt;
  pg_tt_find(d, g, s->stream);
  int np = 0;
  TRY(d2h(s, &np, g.np_dev, 1));
  CK(cudaStreamSynchronize(s->stream));
  if (np > g.cap)
  {
    // room for the pairs of this step (and the next): both pair lists grow
    // together, the previous step's list keeping its entries
    const int cap = np + np / 2 + 1024;
    int *ppu = nullptr; unsigned char *pact = nullptr; double *pst[3] = {};
    int *pf = nullptr, *pu = nullptr; unsigned char *act = nullptr; double *st[3] = {}, *f[3] = {}, *p[3] = {};
    int *queue = nullptr;
    TRY(dalloc(s, &pf, cap)); TRY(dalloc(s, &pu, cap)); TRY(dalloc(s, &act, cap)); TRY(dalloc(s, &ppu, cap));
    TRY(dalloc(s, &queue, cap));
    TRY(dalloc(s, &pact, cap));
    for (int c = 0; c < 3; c ++)
    {
      TRY(dalloc(s, &st[c], cap)); TRY(dalloc(s, &f[c], cap)); TRY(dalloc(s, &p[c], cap)); TRY(dalloc(s, &pst[c], cap));
    }
    if (g.cap > 0)
    {
      CK(cudaMemcpyAsync(ppu, g.ppu, (size_t)g.cap * sizeof(int), cudaMemcpyDeviceToDevice, s->stream));
      CK(cudaMemcpyAsync(pact, g.pact, (size_t)g.cap, cudaMemcpyDeviceToDevice, s->stream));
      for (int c = 0; c < 3; c ++)
        CK(cudaMemcpyAsync(pst[c], g.pst[c], (size_t)g.cap * sizeof(double), cudaMemcpyDeviceToDevice, s->stream));
    }
    CK(cudaStreamSynchronize(s->stream));
    for (void *q : {(void *)g.pf, (void *)g.pu, (void *)g.act, (void *)g.ppu, (void *)g.pact, (void *)g.queue})
      release(s, q);
    for (int c = 0; c < 3; c ++) for (void *q : {(void *)g.st[c], (void *)g.f[c], (void *)g.p[c], (void *)g.pst[c]}) release(s, q);
    release(s, g.ekeys[0]); release(s, g.ekeys[1]); release(s, g.evals[0]); release(s, g.evals[1]); release(s, g.ehist);
    TRY(dalloc(s, &g.ekeys[0], 2 * (size_t)cap)); TRY(dalloc(s, &g.ekeys[1], 2 * (size_t)cap));
    TRY(dalloc(s, &g.evals[0], 2 * (size_t)cap)); TRY(dalloc(s, &g.evals[1], 2 * (size_t)cap));
    TRY(dalloc(s, &g.ehist, pg_sort_hist_len(2 * cap)));
    g.pf = pf; g.pu = pu; g.act = act; g.ppu = ppu; g.pact = pact; g.queue = queue;
    for (int c = 0; c < 3; c ++) { g.st[c] = st[c]; g.f[c] = f[c]; g.p[c] = p[c]; g.pst[c] = pst[c]; }
    g.cap = cap;
  }
  const long long chunks = pg_tt_max_chunks(d.parnum, np);
  if (chunks > g.ccap)
  {
    const long long cap = chunks + chunks / 2;
    CK(cudaStreamSynchronize(s->stream));
    for (int c = 0; c < 6; c ++)
    {
      release(s, g.csum[c]);
      g.csum[c] = nullptr;
      TRY(dalloc(s, &g.csum[c], (size_t)cap));
    }
    g.ccap = cap;
  }
  pg_tt_forces(d, g, s->stream, np, step);
  s->launches += pg_tt_kernel_count(g, d.trinum, np);
  // this step's pairs become the previous step's
  g.np_last = np;
  std::swap(g.off, g.poff);
  std::swap(g.pu, g.ppu);
  std::swap(g.act, g.pact);
  for (int c = 0; c < 3; c ++) std::swap(g.st[c], g.pst[c]);
  CK(cudaGetLastError());
  return PG_OK;
}

// capture one step into a CUDA graph (kernel arguments are baked in: the
// graph is re-captured when a buffer is reallocated or the step changes)
int capture_step(pg_session *s, double step)
{
  if (s->graph_exec && !s->graph_adapt && s->graph_step == step) return PG_OK;
  drop_graph(s);
  CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  enqueue_step(s, step);
  CK(cudaStreamEndCapture(s->stream, &s->graph));
  CK(cudaGraphInstantiate(&s->graph_exec, s->graph, 0));
  s->graph_step = step;
  s->graph_adapt = 0;
  return PG_OK;
}

// PG_GRAPH_STEPS steps as one graph, for the step of the current one-step graph
int capture_steps(pg_session *s, double step)
{
  TRY(capture_step(s, step));
  if (s->graphn_exec) return PG_OK;
  CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  for (int k = 0; k < PG_GRAPH_STEPS; k ++) enqueue_step(s, step);
  CK(cudaStreamEndCapture(s->stream, &s->graphn));
  CK(cudaGraphInstantiate(&s->graphn_exec, s->graphn, 0));
  return PG_OK;
}

void enqueue_step_adaptive(pg_session *s);

int capture_step_adaptive(pg_session *s)
{
  if (s->graph_exec && s->graph_adapt) return PG_OK;
  drop_graph(s);
  CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  enqueue_step_adaptive(s);
  CK(cudaStreamEndCapture(s->stream, &s->graph));
  CK(cudaGraphInstantiate(&s->graph_exec, s->graph, 0));
  s->graph_adapt = 1;
  return PG_OK;
}

// per-particle and per-spring stiffness terms, the step pair and the
// per-step records (sized with the step tables)
int adapt_buffers(pg_session *s)
{
  PgDev &d = s->d;
  const size_t P = std::max(d.parnum, 1), S = std::max(d.sprnum, 1);
  if (!s->adapt_ready)
  {
    for (int k = 0; k < 3; k ++) TRY(dalloc(s, &d.akact[k], P));
    for (int k = 0; k < 6; k ++) TRY(dalloc(s, &d.akrot[k], P));
    TRY(dalloc(s, &d.akmax, P));
    TRY(dalloc(s, &d.aemax, P));
    for (int k = 0; k < 17; k ++) TRY(dalloc(s, &d.sad[k], S));
    for (int k = 0; k < 3; k ++) TRY(dalloc(s, &d.tq_k[k], (size_t)std::max(d.trqsprnum, 1)));
    TRY(dalloc(s, &s->hs_buf, 4));
    TRY(dalloc(s, &d.hmin, 1));
    const unsigned long long big = 0x7fefffffffffffffull;
    TRY(h2d(s, d.hmin, &big, 1));
    s->adapt_ready = 1;
  }
  if (s->sbig_ad_cap < std::max(d.nbig, 1))
  {
    drop_graph(s);
    CK(cudaStreamSynchronize(s->stream));
    release(s, d.sbig_ad);
    d.sbig_ad = nullptr;
    TRY(dalloc(s, &d.sbig_ad, 11 * (size_t)std::max(d.nbig, 1)));
    s->sbig_ad_cap = std::max(d.nbig, 1);
  }
  if (s->hrec_cap < s->tab_cap)
  {
    drop_graph(s);
    CK(cudaStreamSynchronize(s->stream));
    release(s, d.hrec);
    d.hrec = nullptr;
    TRY(dalloc(s, &d.hrec, (size_t)s->tab_cap));
    s->hrec_cap = s->tab_cap;
  }
  return PG_OK;
}

// one adaptive step: forces with the stiffness terms, the step choice on
// the device, then the rest of the step with (step0, step1) from d.hs
void enqueue_step_adaptive(pg_session *s)
{
  const PgDev &d = s->d;
  pg_launch_rebuild(d, s->stream);
  pg_launch_excite(d, s->stream, 0.0);
  pg_launch_contacts(d, s->stream, 0.0);
  pg_launch_springs(d, s->stream, 0.0);
  pg_launch_spring_runs(d, s->stream);
  pg_launch_torsion(d, s->stream, 0.0);
  pg_launch_unspring(d, s->stream);
  pg_launch_force_sums_adapt(d, s->stream);
  pg_launch_adapt_step(d, s->stream);
  pg_launch_dynamics_fused(d, s->stream);
  pg_launch_mesh(d, s->stream);
  pg_launch_obstacles_tail(d, s->stream, 0.0);
}

int adaptive_kernel_count(const PgDev &d)
{
  int n = pg_rebuild_kernel_count(d) + 2 + 1;     // excite, select, tail
  if (d.ellnum) n += 1;
  if (d.sprnum) n += 1 + (d.nbig > 0 ? 4 : 0) + (d.unsprnum ? 1 : 0);
  if (d.trqsprnum) n += 1;
  if (d.parnum) n += 3;                           // force sums, minimum, dynamics
  if (d.nodnum) n += 1;
  if (d.facnum) n += 1;
  if (d.obsnum && d.trinum) n += 1;
  return n;
}

// host step tables of one call -> device (rows [0, n))
int upload_tables(pg_session *s, const pg_steptab *tab, int n)
{
  PgDev &d = s->d;
  std::vector<double> zeros;
  auto put = [&](double *dst, const double *src, size_t width) -> int {
    if (src) return h2d(s, dst, src, (size_t)n * width);
    zeros.assign((size_t)n * width, 0.0);
    int r = h2d(s, dst, zeros.data(), (size_t)n * width);
    if (r == PG_OK && cudaStreamSynchronize(s->stream) != cudaSuccess) return PG_ERR_CUDA;
    return r;
  };
  TRY(put(d.t_curtime, tab->curtime, 1));
  TRY(put(d.t_gravity, tab->gravity, 3));
  TRY(put(d.t_damping, tab->damping, 6));
  TRY(put(d.t_prs_lin, tab->prs_lin, s->prs_stride));
  TRY(put(d.t_prs_ang, tab->prs_ang, s->prs_stride));
  TRY(put(d.t_obs_ang, tab->obs_ang, s->obs_stride));
  TRY(put(d.t_obs_lin, tab->obs_lin, s->obs_stride));
  CK(cudaMemsetAsync(d.stepno, 0, sizeof(int), s->stream));
  if (d.ustep) TRY(h2d(s, d.ustep, &tab->stepnum, 1));
  return PG_OK;
}

int read_err(pg_session *s)
{
  int e = 0;
  CK(cudaMemcpyAsync(&e, s->d.err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return e;
}

} // namespace

extern "C" {

const char *pg_version(void) { return "parmec_gb300 0.1.0 (sm_103a)"; }

int pg_session_create(const pg_scene *sc, int form, pg_session **out)
{
  if (!sc || !out || sc->parnum < 0 || sc->ellnum < 0) return PG_ERR_ARGUMENT;
  if (form != PG_FORM_FP64 && form != PG_FORM_MIXED) return PG_ERR_ARGUMENT;
  if (form == PG_FORM_MIXED)
  {
    // scope of the mixed form: spheres centred on their particle, obstacles, analytical particles
    if (sc->sprnum || sc->nodnum || sc->facnum || sc->rstnum > 0 || sc->trqsprnum > 0 || sc->pbfnum > 0)
      return PG_ERR_UNSUPPORTED;
    for (int e = 0; e < sc->ellnum; e ++)
    {
      int p = sc->part[e];
      for (int k = 0; k < 3; k ++)
        if (sc->center[3+k][e] != sc->position[3+k][p]) return PG_ERR_UNSUPPORTED;
    }
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return PG_ERR_CUDA;
  pg_session *s = new pg_session();
  std::memset(&s->d, 0, sizeof(PgDev));
  PgDev &d = s->d;
  int r = PG_OK;
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) { delete s; return PG_ERR_CUDA; }
  d.parnum = sc->parnum; d.ellnum = sc->ellnum; d.trinum = sc->trinum; d.obsnum = sc->obsnum;
  d.estride = d.ellnum;
  d.nodnum = sc->nodnum; d.facnum = sc->facnum; d.sprnum = sc->sprnum; d.pairnum = sc->pairnum;
  d.prsnum = sc->prsnum; d.compat = sc->compat; d.form = form;
  d.nscene = sc->nscene > 0 ? sc->nscene : 1;
  d.kn = 32; d.kr = 32;
  s->prs_stride = 3 * std::max(1, sc->prsnum);
  s->obs_stride = 3 * std::max(1, sc->obsnum);
  d.tab_prs_stride = s->prs_stride;
  d.tab_obs_stride = s->obs_stride;
  if ((r = allocate(s, sc)) != PG_OK) goto fail;
  if ((r = dalloc(s, &d.stepno, 1)) != PG_OK) goto fail;
  if ((r = dalloc(s, &d.rebuild, 1)) != PG_OK) goto fail;
  if ((r = dalloc(s, &d.obs_done, 1)) != PG_OK) goto fail;
  if ((r = dalloc(s, &d.err, 4)) != PG_OK) goto fail;
  if ((r = dalloc(s, &d.stats, 8)) != PG_OK) goto fail;
  if ((r = contact_buffers(s)) != PG_OK) goto fail;
  if (form == PG_FORM_MIXED && (r = mixed_buffers(s)) != PG_OK) goto fail;
  if ((r = upload_static(s, sc)) != PG_OK) goto fail;
  if ((r = upload_all(s, sc)) != PG_OK) goto fail;
  if ((r = grid_from_scene(s, sc)) != PG_OK) goto fail;
  if ((r = ensure_tables(s, 64)) != PG_OK) goto fail;
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) { r = PG_ERR_CUDA; goto fail; }
  *out = s;
  return PG_OK;
fail:
  pg_session_destroy(s);
  return r;
}

int pg_session_destroy(pg_session *s)
{
  if (!s) return PG_OK;
  if (s->stream) cudaStreamSynchronize(s->stream);
  drop_graph(s);
  for (void *p : s->allocs) cudaFree(p);
  for (auto &e : s->ring) if (e) cudaEventDestroy(e);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return PG_OK;
}

int pg_session_set_skin(pg_session *s, double skin)
{
  if (!s) return PG_ERR_ARGUMENT;
  s->d.skin = skin > 0.0 ? skin : 0.0;
  const double cell_old = s->d.cell;
  pg_rebuild_grid_params(s->d, s->ext, s->rmax, s->rmin);
  for (auto &o : s->sorg_h) o += 4.0 * (cell_old - s->d.cell);
  return grid_buffers(s);
}

int pg_session_record_geometry(pg_session *s, int on)
{
  if (!s) return PG_ERR_ARGUMENT;
  s->d.record_geometry = on ? 1 : 0;
  drop_graph(s);
  return PG_OK;
}

int pg_session_upload(pg_session *s, const pg_scene *sc)
{
  if (!s || !sc) return PG_ERR_ARGUMENT;
  if (sc->parnum != s->d.parnum || sc->ellnum != s->d.ellnum || sc->trinum != s->d.trinum ||
      sc->sprnum != s->d.sprnum || sc->obsnum != s->d.obsnum || sc->prsnum != s->d.prsnum)
    return PG_ERR_ARGUMENT;
  if (s->d.compat != sc->compat) drop_graph(s);
  s->d.compat = sc->compat;
  TRY(upload_all(s, sc));
  if (sc->unsprnum == s->d.unsprnum && s->d.unsprnum) TRY(h2d(s, s->d.nfreq, sc->nfreq, s->d.unsprnum));
  CK(cudaStreamSynchronize(s->stream));
  return PG_OK;
}

int pg_session_invert_inertia(pg_session *s)
{
  if (!s) return PG_ERR_ARGUMENT;
  pg_launch_invert(s->d, s->stream);
  s->launches += 1;
  if (s->d.form == PG_FORM_MIXED) { pg_launch_mx_inertia(s->d, s->stream); s->launches += 1; }
  CK(cudaGetLastError());
  return PG_OK;
}

int pg_session_first_half_step(pg_session *s, double step, const double *obs_ang, const double *obs_lin)
{
  if (!s) return PG_ERR_ARGUMENT;
  PgDev &d = s->d;
  if (d.form == PG_FORM_MIXED) pg_launch_mx_to64(d, s->stream);
  pg_launch_euler(d, s->stream, 0.5 * step);
  pg_launch_shapes(d, s->stream, false);
  if (d.obsnum)
  {
    TRY(h2d(s, d.obsang, obs_ang, 3 * (size_t)d.obsnum));
    TRY(h2d(s, d.obslin, obs_lin, 3 * (size_t)d.obsnum));
  }
  pg_launch_obstacles_state(d, s->stream, step);
  s->launches += 5;
  if (d.form == PG_FORM_MIXED) { pg_launch_mx_from64(d, s->stream); s->launches += 2; }
  CK(cudaGetLastError());
  return PG_OK;
}

static int run_steps(pg_session *s, const pg_steptab *tab, double step, bool wait);

int pg_session_run(pg_session *s, const pg_steptab *tab, double step) { return run_steps(s, tab, step, true); }

int pg_session_run_async(pg_session *s, const pg_steptab *tab, double step) { return run_steps(s, tab, step, false); }

// enqueue tab->nsteps steps; with 'wait' return once they finished.  The
// step tables are copied to the device before the first launch (the copies
// from pageable memory are staged by the driver before the call returns), so
// the host tables may change as soon as this returns.
static int run_steps(pg_session *s, const pg_steptab *tab, double step, bool wait)
{
  if (!s || !tab || tab->nsteps < 0) return PG_ERR_ARGUMENT;
  PgDev &d = s->d;
  const int n = tab->nsteps;
  if (n == 0) return PG_OK;
  TRY(ensure_tables(s, n));
  TRY(upload_tables(s, tab, n));
  if (s->fused && d.form == PG_FORM_MIXED && !s->profile)
  {
    const long long before = s->fused_launches;
    TRY(run_fused_steps(s, step, n));
    s->launches += s->fused_launches - before;
    CK(cudaGetLastError());
    if (wait) CK(cudaStreamSynchronize(s->stream));
    return PG_OK;
  }
  const int per_step = pg_rebuild_kernel_count(d) + pg_step_kernel_count(d) + (d.form == PG_FORM_MIXED ? 1 : 0);
  if (!s->profile && s->use_graph && !d.tt_on)
  {
    TRY(capture_step(s, step));
    int k = 0;
    if (n >= PG_GRAPH_STEPS)
    {
      TRY(capture_steps(s, step));
      for (; k + PG_GRAPH_STEPS <= n; k += PG_GRAPH_STEPS) CK(cudaGraphLaunch(s->graphn_exec, s->stream));
    }
    for (; k < n; k ++) CK(cudaGraphLaunch(s->graph_exec, s->stream));
  }
  else if (!s->profile)
  {
    for (int k = 0; k < n; k ++) enqueue_step(s, step);
  }
  else
  {
    // groups: 0 rebuild, 1 contacts, 2 springs, 3 integrate, 4 mesh, 5 obstacles + tail
    const PgDev d = live_view(s);
    const int G = 6;
    s->ring.resize((size_t)n * (G + 1));
    for (auto &e : s->ring) if (!e) CK(cudaEventCreate(&e));
    for (int k = 0; k < n; k ++)
    {
      cudaEvent_t *ev = &s->ring[(size_t)k * (G + 1)];
      CK(cudaEventRecord(ev[0], s->stream));
      if (d.form == PG_FORM_MIXED) pg_launch_mx_centres(d, s->stream);
      pg_launch_rebuild(d, s->stream);
      pg_launch_excite(d, s->stream, step);
      CK(cudaEventRecord(ev[1], s->stream));
      if (d.form == PG_FORM_MIXED) pg_launch_contacts_mx(d, s->stream, step);
      else pg_launch_contacts(d, s->stream, step);
      CK(cudaEventRecord(ev[2], s->stream));
      if (d.form != PG_FORM_MIXED)
      {
        pg_launch_springs(d, s->stream, step);
        pg_launch_spring_runs(d, s->stream);
        pg_launch_torsion(d, s->stream, step);
        pg_launch_unspring(d, s->stream);
        if (d.tt_on) TRY(tt_stage(s, step));
      }
      CK(cudaEventRecord(ev[3], s->stream));
      if (d.form == PG_FORM_MIXED) pg_launch_integrate_mx(d, s->stream, step);
      else pg_launch_integrate(d, s->stream, step);
      CK(cudaEventRecord(ev[4], s->stream));
      pg_launch_mesh(d, s->stream);
      CK(cudaEventRecord(ev[5], s->stream));
      pg_launch_obstacles_tail(d, s->stream, step);
      CK(cudaEventRecord(ev[6], s->stream));
    }
    CK(cudaStreamSynchronize(s->stream));
    const int counts[6] = {pg_rebuild_kernel_count(d), pg_contacts_kernel_count(d), d.sprnum ? 1 : 0, d.parnum ? 1 : 0,
                           (d.nodnum ? 1 : 0) + (d.facnum ? 1 : 0), pg_obstacles_kernel_count(d)};
    for (int k = 0; k < n; k ++)
    {
      cudaEvent_t *ev = &s->ring[(size_t)k * (G + 1)];
      for (int g = 0; g < G; g ++)
      {
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, ev[g], ev[g + 1]));
        s->group_ms[g] += ms;
        s->group_launches[g] += counts[g];
      }
    }
  }
  s->launches += (long long)per_step * n;
  CK(cudaGetLastError());
  if (wait) CK(cudaStreamSynchronize(s->stream));
  return PG_OK;
}

} // extern "C"

namespace {

template <typename T>
int grow_scratch(pg_session *s, T *&p, size_t &cap, size_t n)
{
  if (n <= cap) return PG_OK;
  CK(cudaStreamSynchronize(s->stream));
  release(s, (void *)p);
  p = nullptr;
  cap = 0;
  TRY(dalloc(s, &p, n));
  cap = n;
  return PG_OK;
}

// rows idx[0..n) of ncols device arrays into the matching host arrays
int gather_download(pg_session *s, const double *const *dcols, double *const *hcols, int ncols, const int *idx, int n,
                    int limit)
{
  if (n <= 0 || ncols <= 0) return PG_OK;
  for (int j = 0; j < n; j ++) if (idx[j] < 0 || idx[j] >= limit) return PG_ERR_ARGUMENT;
  TRY(grow_scratch(s, s->g_idx, s->g_idx_cap, (size_t)n));
  TRY(grow_scratch(s, s->g_cols, s->g_cols_cap, (size_t)ncols));
  TRY(grow_scratch(s, s->g_out, s->g_out_cap, (size_t)n * ncols));
  std::vector<double> out((size_t)n * ncols);
  TRY(h2d(s, s->g_idx, idx, (size_t)n));
  TRY(h2d(s, s->g_cols, dcols, (size_t)ncols));
  pg_launch_gather(s->g_cols, ncols, s->g_idx, n, s->g_out, s->stream);
  s->launches += 1;
  CK(cudaGetLastError());
  TRY(d2h(s, out.data(), s->g_out, out.size()));
  CK(cudaStreamSynchronize(s->stream));
  for (int c = 0; c < ncols; c ++)
    if (hcols[c]) for (int j = 0; j < n; j ++) hcols[c][idx[j]] = out[(size_t)c * n + j];
  return PG_OK;
}

} // namespace

extern "C" {

int pg_session_download_particles(pg_session *s, pg_scene *sc, const int *idx, int n)
{
  if (!s || !sc || n < 0 || (n > 0 && !idx)) return PG_ERR_ARGUMENT;
  PgDev &d = s->d;
  if (d.form == PG_FORM_MIXED) pg_launch_mx_to64(d, s->stream);
  const double *dc[30];
  double *hc[30];
  int c = 0;
  for (int k = 0; k < 6; k ++) { dc[c] = d.angular[k]; hc[c ++] = sc->angular[k]; }
  for (int k = 0; k < 3; k ++) { dc[c] = d.linear[k]; hc[c ++] = sc->linear[k]; }
  for (int k = 0; k < 9; k ++) { dc[c] = d.rotation[k]; hc[c ++] = sc->rotation[k]; }
  for (int k = 0; k < 6; k ++) { dc[c] = d.position[k]; hc[c ++] = sc->position[k]; }
  for (int k = 0; k < 3; k ++) { dc[c] = d.force[k]; hc[c ++] = sc->force[k]; }
  for (int k = 0; k < 3; k ++) { dc[c] = d.torque[k]; hc[c ++] = sc->torque[k]; }
  return gather_download(s, dc, hc, c, idx, n, d.parnum);
}

int pg_session_download_springs(pg_session *s, pg_scene *sc, const int *idx, int n)
{
  if (!s || !sc || n < 0 || (n > 0 && !idx)) return PG_ERR_ARGUMENT;
  PgDev &d = s->d;
  const double *dc[12];
  double *hc[12];
  int c = 0;
  for (int a = 0; a < 2; a ++)
    for (int k = 0; k < 3; k ++) { dc[c] = d.sprpnt[6*a+k]; hc[c ++] = sc->sprpnt[a][k]; }
  for (int k = 0; k < 3; k ++) { dc[c] = d.stroke[k]; hc[c ++] = sc->stroke[k]; }
  for (int k = 0; k < 3; k ++) { dc[c] = d.sprfrc[k]; hc[c ++] = sc->sprfrc[k]; }
  return gather_download(s, dc, hc, c, idx, n, d.sprnum);
}

int pg_session_restrain_velocities(pg_session *s)
{
  if (!s) return PG_ERR_ARGUMENT;
  if (s->d.rstnum == 0) return PG_OK;
  pg_launch_restrain_velocities(s->d, s->stream);
  s->launches += 1;
  CK(cudaGetLastError());
  return PG_OK;
}

int pg_session_mesh_contact(pg_session *s, double radius, double cell, const unsigned char *big)
{
  if (!s || !(radius >= 0.0)) return PG_ERR_ARGUMENT;
  PgDev &d = s->d;
  if (radius == 0.0) { d.tt_on = 0; return PG_OK; }
  if (!(cell > 0.0) || !big) return PG_ERR_ARGUMENT;
  if (d.form != PG_FORM_FP64 || d.nscene > 1) return PG_ERR_UNSUPPORTED;
  PgTT &g = s->tt;
  const int T = d.trinum, P = d.parnum;
  if (T <= 0 || P <= 0) return PG_OK;
  drop_graph(s);
  CK(cudaStreamSynchronize(s->stream));
  // the grid spans the mesh triangles' present boxes with two cells of
  // margin each way (triangles that leave it take the nearest cell: only
  // the search slows, no pair is lost)
  std::vector<double> tri(9 * (size_t)T);
  std::vector<int> tob(T);
  for (int k = 0; k < 9; k ++) TRY(d2h(s, tri.data() + (size_t)k * T, d.tri[k], T));
  TRY(d2h(s, tob.data(), d.triobs, T));
  CK(cudaStreamSynchronize(s->stream));
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int t = 0; t < T; t ++)
  {
    if (tob[t] < 0 || big[t]) continue;
    for (int a = 0; a < 3; a ++)
      for (int c = 0; c < 3; c ++)
      {
        const double x = tri[(size_t)(3*a + c) * T + t];
        lo[c] = std::min(lo[c], x);
        hi[c] = std::max(hi[c], x);
      }
  }
  double h = cell;
  for (int c = 0; c < 3; c ++) if (!(hi[c] >= lo[c])) { lo[c] = 0.0; hi[c] = 0.0; }
  long long cells = 0;
  int dim[3];
  for (;;)
  {
    cells = 1;
    for (int c = 0; c < 3; c ++)
    {
      dim[c] = (int)std::ceil((hi[c] - lo[c]) / h) + 5;
      cells *= dim[c];
    }
    if (cells <= (1LL << 26)) break;
    h *= 1.25;                                 // a coarser grid: more triangles per cell, the same pairs
  }
  g.r = radius;
  g.h = h;
  for (int c = 0; c < 3; c ++) { g.org[c] = lo[c] - 2.0 * h; g.dim[c] = dim[c]; }
  g.ncells = (int)cells;
  const int kb = pg_tt_key_bits(g.ncells);
  g.none = (1u << kb) - 1u;
  g.passes = pg_sort_passes_bits(kb);
  int pb = 1;
  while ((1u << pb) <= (unsigned)P) pb ++;
  g.enone = (1u << pb) - 1u;
  g.epasses = pg_sort_passes_bits(pb);
  if (!g.big)
  {
    TRY(dalloc(s, &g.big, T));
    for (int c = 0; c < 6; c ++) TRY(dalloc(s, &g.box[c], T));
    TRY(dalloc(s, &g.cell, T));
    for (int k = 0; k < 2; k ++) { TRY(dalloc(s, &g.keys[k], T)); TRY(dalloc(s, &g.vals[k], T)); }
    TRY(dalloc(s, &g.hist, pg_sort_hist_len(T)));
    TRY(dalloc(s, &g.cand, (size_t)g.kmax * T));
    TRY(dalloc(s, &g.cnt, T));
    TRY(dalloc(s, &g.off, (size_t)T + 1));
    TRY(dalloc(s, &g.poff, (size_t)T + 1));
    TRY(dalloc(s, &g.np_dev, 1));
    TRY(dalloc(s, &g.pfirst, P));
    TRY(dalloc(s, &g.plast, P));
    TRY(dalloc(s, &g.nch, P));
    TRY(dalloc(s, &g.choff, (size_t)P + 1));
    TRY(dalloc(s, &g.nchunks, 1));
    TRY(dalloc(s, &g.qn, 1));
    for (int c = 0; c < 3; c ++) { TRY(dalloc(s, &d.ttF[c], P)); TRY(dalloc(s, &d.ttT[c], P)); }
  }
  release(s, g.cstart);
  release(s, g.cend);
  TRY(dalloc(s, &g.cstart, (size_t)g.ncells + 1));
  TRY(dalloc(s, &g.cend, (size_t)g.ncells + 1));
  TRY(h2d(s, g.big, big, T));
  // no pairs carried into the first step
  CK(cudaMemsetAsync(g.poff, 0, ((size_t)T + 1) * sizeof(int), s->stream));
  CK(cudaStreamSynchronize(s->stream));
  d.tt_on = 1;
  return PG_OK;
}

int pg_session_set_live(pg_session *s, int particles, int spheres, int triangles)
{
  if (!s) return PG_ERR_ARGUMENT;
  PgDev &d = s->d;
  if (particles < 0 || spheres < 0 || triangles < 0 || particles > d.parnum || spheres > d.ellnum ||
      triangles > d.trinum)
    return PG_ERR_ARGUMENT;
  const bool whole = particles == d.parnum && spheres == d.ellnum && triangles == d.trinum;
  const int e_now = s->elive > 0 ? s->elive : d.ellnum;
  drop_graph(s);
  if (s->fgraph_exec) { cudaGraphExecDestroy(s->fgraph_exec); s->fgraph_exec = nullptr; }
  if (s->fgraph) { cudaGraphDestroy(s->fgraph); s->fgraph = nullptr; }
  CK(cudaStreamSynchronize(s->stream));
  // a rebuild clears the cells of the spheres it sorted last time: cells
  // of spheres beyond a smaller extent would keep stale ranges, so the whole
  // cell table starts empty
  if (spheres < e_now && s->ncells)
  {
    CK(cudaMemsetAsync(d.cstart, 0, s->ncells * sizeof(int), s->stream));
    CK(cudaMemsetAsync(d.cend, 0, s->ncells * sizeof(int), s->stream));
  }
  s->plive = whole ? 0 : particles;
  s->elive = whole ? 0 : spheres;
  s->tlive = whole ? 0 : triangles;
  int one = 1;
  TRY(h2d(s, d.rebuild, &one, 1));
  CK(cudaStreamSynchronize(s->stream));
  return PG_OK;
}

int pg_session_mesh_contact_stats(pg_session *s, int *pairs, int *active)
{
  if (!s || !pairs || !active) return PG_ERR_ARGUMENT;
  PgTT &g = s->tt;
  *pairs = s->d.tt_on ? g.np_last : 0;
  *active = 0;
  if (*pairs > 0)
  {
    std::vector<unsigned char> a(*pairs);
    TRY(d2h(s, a.data(), g.pact, a.size()));
    CK(cudaStreamSynchronize(s->stream));
    for (unsigned char v : a) *active += v ? 1 : 0;
  }
  return PG_OK;
}

int pg_session_critical(pg_session *s, int which, double *h, double *omega, double *ratio)
{
  if (!s || (which != 0 && which != 1)) return PG_ERR_ARGUMENT;
  PgDev &d = s->d;
  if (d.form != PG_FORM_FP64) return PG_ERR_UNSUPPORTED;
  const size_t P = std::max(d.parnum, 1), S = std::max(d.sprnum, 1);
  if (!s->crit_h)
  {
    TRY(adapt_buffers(s));
    TRY(dalloc(s, &s->crit_ke, 2 * S));
    TRY(dalloc(s, &s->crit_h, std::max(P, S)));
    TRY(dalloc(s, &s->crit_o, std::max(P, S)));
    TRY(dalloc(s, &s->crit_r, std::max(P, S)));
  }
  size_t n;
  if (which == 0)
  {
    pg_launch_critical_perparticle(d, s->stream, s->crit_ke, 1, s->crit_h, s->crit_o, s->crit_r);
    s->launches += d.sprnum ? 2 : 1;
    n = d.parnum;
  }
  else
  {
    pg_launch_critical_perspring(d, s->stream, s->crit_h, s->crit_o, s->crit_r);
    s->launches += d.sprnum ? 1 : 0;
    n = d.sprnum;
  }
  CK(cudaGetLastError());
  TRY(d2h(s, h, s->crit_h, n));
  TRY(d2h(s, omega, s->crit_o, n));
  TRY(d2h(s, ratio, s->crit_r, n));
  CK(cudaStreamSynchronize(s->stream));
  return PG_OK;
}

int pg_session_run_adaptive(pg_session *s, const pg_steptab *tab, double step0, double adaptive, double *steps)
{
  if (!s || !tab || tab->nsteps < 0 || !(adaptive > 0.0 && adaptive <= 1.0) || !(step0 > 0.0))
    return PG_ERR_ARGUMENT;
  PgDev &d = s->d;
  if (d.form != PG_FORM_FP64 || d.nscene > 1 || s->exc_any || d.tt_on) return PG_ERR_UNSUPPORTED;
  const int n = tab->nsteps;
  if (n == 0) return PG_OK;
  TRY(ensure_tables(s, n));
  TRY(adapt_buffers(s));
  TRY(upload_tables(s, tab, n));
  const double h3[3] = {step0, step0, adaptive};
  TRY(h2d(s, s->hs_buf, h3, 3));
  d.hs = s->hs_buf;
  int rc = PG_OK;
  if (s->use_graph && !s->profile)
  {
    rc = capture_step_adaptive(s);
    for (int k = 0; k < n && rc == PG_OK; k ++)
      if (cudaGraphLaunch(s->graph_exec, s->stream) != cudaSuccess) rc = PG_ERR_CUDA;
  }
  else for (int k = 0; k < n; k ++) enqueue_step_adaptive(s);
  d.hs = nullptr;
  TRY(rc);
  s->launches += (long long)adaptive_kernel_count(d) * n;
  CK(cudaGetLastError());
  if (steps) TRY(d2h(s, steps, d.hrec, (size_t)n));
  CK(cudaStreamSynchronize(s->stream));
  return PG_OK;
}

int pg_session_sync(pg_session *s)
{
  if (!s) return PG_ERR_ARGUMENT;
  CK(cudaStreamSynchronize(s->stream));
  int e = read_err(s);
  return e ? e : PG_OK;
}

int pg_session_download(pg_session *s, pg_scene *sc)
{
  if (!s || !sc) return PG_ERR_ARGUMENT;
  PgDev &d = s->d;
  const size_t N = d.nodnum, S = d.sprnum;
  TRY(download_ranges(s, sc, full_ranges(d)));
  for (int k = 0; k < 3; k ++) TRY(d2h(s, sc->nodes[k], d.nodes[k], N));
  TRY(d2h(s, sc->unspring, d.unspring, S));
  if (d.unsprnum && sc->nfreq && sc->unsprnum == d.unsprnum) TRY(d2h(s, sc->nfreq, d.nfreq, d.unsprnum));
  TRY(torsion_state(s, sc, false));
  if (d.pbfnum && sc->pbfnum == d.pbfnum)
    for (int c = 0; c < 6; c ++) TRY(d2h(s, sc->pbfin[c], d.pbfin[c], (size_t)d.pbfnum));
  for (int a = 0; a < 2; a ++)
    for (int k = 0; k < 3; k ++) TRY(d2h(s, sc->sprpnt[a][k], d.sprpnt[6*a+k], S));
  for (int k = 0; k < 2; k ++) TRY(d2h(s, sc->yield[k], d.yield[k], S));
  for (int k = 0; k < 3; k ++) TRY(d2h(s, sc->sprdir[k], d.sprdir[k], S));
  TRY(d2h(s, sc->sprflg, d.sprflg, S));
  for (int k = 0; k < 3; k ++)
  {
    TRY(d2h(s, sc->sprsdsp[k], d.sprsdsp[k], S));
    TRY(d2h(s, sc->stroke[k], d.stroke[k], S));
    TRY(d2h(s, sc->sprfrc[k], d.sprfrc[k], S));
  }
  CK(cudaStreamSynchronize(s->stream));
  int e = read_err(s);
  return e ? e : PG_OK;
}

int pg_session_set_capacity(pg_session *s, int kn, int kr)
{
  if (!s || kn < 1 || kr < 1 || kn > 96 || kr > 96) return PG_ERR_ARGUMENT;
  PgDev &d = s->d;
  CK(cudaStreamSynchronize(s->stream));
  drop_graph(s);
  release_slot_buffers(s);
  d.kn = kn;
  d.kr = kr;
  TRY(slot_buffers(s));
  if (d.ellnum) CK(cudaMemsetAsync(d.ncnt, 0, (size_t)d.ellnum * sizeof(int), s->stream));
  int one = 1;
  TRY(h2d(s, d.rebuild, &one, 1));
  CK(cudaStreamSynchronize(s->stream));
  return PG_OK;
}

int pg_session_set_grid(pg_session *s, double cell, const int dim[3])
{
  if (!s || !dim || !(cell > 0.0)) return PG_ERR_ARGUMENT;
  for (int k = 0; k < 3; k ++) if (dim[k] < 1 || dim[k] > 512) return PG_ERR_ARGUMENT;
  PgDev &d = s->d;
  if (cell < 2.0 * s->rmax + d.skin) return PG_ERR_ARGUMENT;   // neighbours must lie in adjacent cells
  d.cell = cell;
  for (int k = 0; k < 3; k ++) d.dim[k] = dim[k];
  pg_rebuild_key_bits(d);
  return grid_buffers(s);
}

int pg_session_scene(pg_session *s, int scene, int active, const double origin[3], const double exc[PG_EXC_LEN],
                     long long start_step)
{
  if (!s || scene < 0 || scene >= s->d.nscene) return PG_ERR_ARGUMENT;
  PgDev &d = s->d;
  int a = active ? 1 : 0, on = exc ? 1 : 0;
  if (exc) s->exc_any = 1;
  TRY(h2d(s, d.sactive + scene, &a, 1));
  TRY(h2d(s, d.sexc_on + scene, &on, 1));
  if (exc) TRY(h2d(s, d.sexc + (size_t)PG_EXC_LEN * scene, exc, PG_EXC_LEN));
  if (origin)
    for (int k = 0; k < 3; k ++)
    {
      s->sorg_h[(size_t)k * d.nscene + scene] = origin[k];
      TRY(h2d(s, d.sorg[k] + scene, &origin[k], 1));
    }
  long long st = start_step;
  if (st < 0) CK(cudaMemcpyAsync(d.sstart + scene, d.gstep, sizeof(long long), cudaMemcpyDeviceToDevice, s->stream));
  else TRY(h2d(s, d.sstart + scene, &st, 1));
  int one = 1;
  TRY(h2d(s, d.rebuild, &one, 1));
  CK(cudaStreamSynchronize(s->stream));
  return PG_OK;
}

static int ranges_of(const PgDev &d, const int *r, Ranges *out)
{
  if (!r) return PG_ERR_ARGUMENT;
  const int lim[4] = {d.parnum, d.ellnum, d.trinum, d.obsnum};
  for (int k = 0; k < 4; k ++)
    if (r[2*k] < 0 || r[2*k+1] < r[2*k] || r[2*k+1] > lim[k]) return PG_ERR_ARGUMENT;
  *out = {(size_t)r[0], (size_t)r[1], (size_t)r[2], (size_t)r[3], (size_t)r[4], (size_t)r[5], (size_t)r[6], (size_t)r[7]};
  return PG_OK;
}

int pg_session_upload_range(pg_session *s, const pg_scene *sc, const int range[8])
{
  if (!s || !sc) return PG_ERR_ARGUMENT;
  Ranges r;
  TRY(ranges_of(s->d, range, &r));
  TRY(upload_ranges(s, sc, r, false, true));
  CK(cudaStreamSynchronize(s->stream));
  return PG_OK;
}

int pg_session_release_range(pg_session *s, const int range[8])
{
  if (!s) return PG_ERR_ARGUMENT;
  PgDev &d = s->d;
  Ranges r;
  TRY(ranges_of(d, range, &r));
  // scene id -1 (all bits set) marks a free entry, which every kernel skips
  if (r.p1 > r.p0) CK(cudaMemsetAsync(d.pscene + r.p0, 0xff, (r.p1 - r.p0) * sizeof(int), s->stream));
  if (r.e1 > r.e0) CK(cudaMemsetAsync(d.escene + r.e0, 0xff, (r.e1 - r.e0) * sizeof(int), s->stream));
  if (r.t1 > r.t0) CK(cudaMemsetAsync(d.tscene + r.t0, 0xff, (r.t1 - r.t0) * sizeof(int), s->stream));
  if (r.o1 > r.o0) CK(cudaMemsetAsync(d.oscene + r.o0, 0xff, (r.o1 - r.o0) * sizeof(int), s->stream));
  if (r.e1 > r.e0) CK(cudaMemsetAsync(d.ncnt + r.e0, 0, (r.e1 - r.e0) * sizeof(int), s->stream));
  int one = 1;
  TRY(h2d(s, d.rebuild, &one, 1));
  CK(cudaStreamSynchronize(s->stream));
  return PG_OK;
}

int pg_session_download_range(pg_session *s, pg_scene *sc, const int range[8])
{
  if (!s || !sc) return PG_ERR_ARGUMENT;
  Ranges r;
  TRY(ranges_of(s->d, range, &r));
  TRY(download_ranges(s, sc, r));
  CK(cudaStreamSynchronize(s->stream));
  int e = read_err(s);
  return e ? e : PG_OK;
}

int pg_session_download_range_motion(pg_session *s, pg_scene *sc, const int range[8])
{
  if (!s || !sc) return PG_ERR_ARGUMENT;
  Ranges r;
  TRY(ranges_of(s->d, range, &r));
  PgDev &d = s->d;
  if (d.form == PG_FORM_MIXED) pg_launch_mx_to64(d, s->stream, (int)r.p0, (int)r.p1);
  for (int k = 0; k < 6; k ++) TRY(d2hr(s, sc->angular[k], d.angular[k], r.p0, r.p1));
  for (int k = 0; k < 3; k ++) TRY(d2hr(s, sc->linear[k], d.linear[k], r.p0, r.p1));
  for (int k = 0; k < 6; k ++) TRY(d2hr(s, sc->position[k], d.position[k], r.p0, r.p1));
  CK(cudaStreamSynchronize(s->stream));
  int e = read_err(s);
  return e ? e : PG_OK;
}

int pg_session_global_step(pg_session *s, long long *step)
{
  if (!s || !step) return PG_ERR_ARGUMENT;
  TRY(d2h(s, step, s->d.gstep, 1));
  CK(cudaStreamSynchronize(s->stream));
  return PG_OK;
}

int pg_session_contact_count(pg_session *s, int *count)
{
  if (!s || !count) return PG_ERR_ARGUMENT;
  PgDev &d = s->d;
  const size_t E = d.ellnum;
  *count = 0;
  if (!E) return PG_OK;
  std::vector<int> cnt(E);
  std::vector<unsigned char> flag((size_t)d.kn * E);
  TRY(d2h(s, cnt.data(), d.ncnt, E));
  TRY(d2h(s, flag.data(), d.nflag, (size_t)d.kn * E));
  CK(cudaStreamSynchronize(s->stream));
  int n = 0;
  for (size_t i = 0; i < E; i ++)
    for (int k = 0; k < cnt[i]; k ++) n += flag[(size_t)k * E + i] ? 1 : 0;
  *count = n;
  return PG_OK;
}

int pg_session_contacts(pg_session *s, int cap, int *count, int *master_particle, int *code,
                        double *point, double *normal, double *depth, double *force, double *state)
{
  if (!s || !count) return PG_ERR_ARGUMENT;
  PgDev &d = s->d;
  const size_t E = d.ellnum, slots = (size_t)d.kn * E;
  *count = 0;
  if (!E) return PG_OK;
  std::vector<int> cnt(E), cod(slots);
  std::vector<unsigned char> flag(slots);
  std::vector<double> st[3], fr[3], pt[3], nr[3], dp(slots);
  TRY(d2h(s, cnt.data(), d.ncnt, E));
  TRY(d2h(s, cod.data(), d.ncode, slots));
  TRY(d2h(s, flag.data(), d.nflag, slots));
  for (int k = 0; k < 3; k ++)
  {
    st[k].resize(slots); fr[k].resize(slots); pt[k].resize(slots); nr[k].resize(slots);
    if (d.form == PG_FORM_MIXED)
    {
      std::vector<float> a(slots), b(slots);
      TRY(d2h(s, a.data(), d.nstate_f[k], slots));
      TRY(d2h(s, b.data(), d.nfrc_f[k], slots));
      CK(cudaStreamSynchronize(s->stream));
      for (size_t q = 0; q < slots; q ++) { st[k][q] = a[q]; fr[k][q] = b[q]; pt[k][q] = nr[k][q] = NAN; }
      continue;
    }
    TRY(d2h(s, st[k].data(), d.nstate[k], slots));
    TRY(d2h(s, fr[k].data(), d.nfrc[k], slots));
    TRY(d2h(s, pt[k].data(), d.npnt[k], slots));
    TRY(d2h(s, nr[k].data(), d.nnrm[k], slots));
  }
  if (d.ndep) TRY(d2h(s, dp.data(), d.ndep, slots));
  else std::fill(dp.begin(), dp.end(), NAN);
  CK(cudaStreamSynchronize(s->stream));
  int n = 0;
  for (int p = 0; p < d.parnum; p ++)
  {
    int i = s->h_pell[p];
    if (i < 0) continue;
    for (int k = 0; k < cnt[i]; k ++)
    {
      size_t idx = (size_t)k * E + i;
      if (!flag[idx]) continue;
      if (n >= cap) { *count = n; return PG_OK; }
      if (master_particle) master_particle[n] = p;
      if (code) code[n] = cod[idx];
      for (int c = 0; c < 3; c ++)
      {
        if (point) point[3*n+c] = pt[c][idx];
        if (normal) normal[3*n+c] = nr[c][idx];
        if (force) force[3*n+c] = fr[c][idx];
        if (state) state[3*n+c] = st[c][idx];
      }
      if (depth) depth[n] = dp[idx];
      n ++;
    }
  }
  *count = n;
  return PG_OK;
}

int pg_session_stream(pg_session *s, void **stream)
{
  if (!s || !stream) return PG_ERR_ARGUMENT;
  *stream = (void *)s->stream;
  return PG_OK;
}

int pg_session_use_graph(pg_session *s, int on)
{
  if (!s) return PG_ERR_ARGUMENT;
  s->use_graph = on ? 1 : 0;
  return PG_OK;
}

int pg_session_use_fused(pg_session *s, int on)
{
  if (!s) return PG_ERR_ARGUMENT;
  if (on && s->d.form != PG_FORM_MIXED) return PG_ERR_UNSUPPORTED;
  CK(cudaStreamSynchronize(s->stream));
  drop_graph(s);
  s->fused = on ? 1 : 0;
  if (on && s->fcfg.shape < 0)
  {
    // default before tuning: 256 threads, as many blocks as fit, fewest spills
    PgFusedCfg buf[32];
    const int m = pg_fused_candidates(buf, 32);
    if (m <= 0) return PG_ERR_CUDA;
    s->fcfg = buf[0];
    for (int k = 0; k < m; k ++) if (buf[k].threads == 256 && buf[k].blocks > s->fcfg.blocks) s->fcfg = buf[k];
  }
  return PG_OK;
}

int pg_session_autotune(pg_session *s, int on)
{
  if (!s) return PG_ERR_ARGUMENT;
  s->tune = on ? 1 : 0;
  s->tuned = 0;
  s->warmed = 0;
  s->cands.clear();
  s->cand_ms.clear();
  return PG_OK;
}

int pg_session_fused_config(pg_session *s, int *out4)
{
  if (!s || !out4) return PG_ERR_ARGUMENT;
  out4[0] = s->fcfg.threads;
  out4[1] = s->fcfg.blocks;
  out4[2] = s->tuned;
  out4[3] = s->fgraph_ok && s->fgraph_exec ? 1 : 0;
  return PG_OK;
}

int pg_session_profile(pg_session *s, int on)
{
  if (!s) return PG_ERR_ARGUMENT;
  s->profile = on ? 1 : 0;
  for (int g = 0; g < 8; g ++) { s->group_ms[g] = 0.0; s->group_launches[g] = 0; }
  return PG_OK;
}

int pg_session_profile_read(pg_session *s, double *ms, long long *launches)
{
  if (!s) return PG_ERR_ARGUMENT;
  for (int g = 0; g < 8; g ++)
  {
    if (ms) ms[g] = s->group_ms[g];
    if (launches) launches[g] = s->group_launches[g];
  }
  return PG_OK;
}

int pg_session_diagnostics(pg_session *s, int *out16)
{
  if (!s || !out16) return PG_ERR_ARGUMENT;
  int e[4], st[8];
  TRY(d2h(s, e, s->d.err, 4));
  TRY(d2h(s, st, s->d.stats, 8));
  CK(cudaStreamSynchronize(s->stream));
  for (int k = 0; k < 4; k ++) out16[k] = e[k];
  for (int k = 0; k < 8; k ++) out16[4 + k] = st[k];
  out16[12] = s->d.dim[0]; out16[13] = s->d.dim[1]; out16[14] = s->d.dim[2]; out16[15] = s->d.bits;
  return PG_OK;
}

int pg_host_register(void *ptr, size_t bytes)
{
  if (!ptr || bytes == 0) return PG_ERR_ARGUMENT;
  cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
  if (e == cudaErrorHostMemoryAlreadyRegistered) { cudaGetLastError(); return PG_OK; }
  if (e != cudaSuccess) { cudaGetLastError(); return PG_ERR_CUDA; }
  return PG_OK;
}

int pg_host_unregister(void *ptr)
{
  if (!ptr) return PG_ERR_ARGUMENT;
  cudaError_t e = cudaHostUnregister(ptr);
  if (e != cudaSuccess) { cudaGetLastError(); return PG_ERR_CUDA; }
  return PG_OK;
}

int pg_session_barrier_selftest(pg_session *s, double *wait_ms)
{
  if (!s) return PG_ERR_ARGUMENT;
  PgDev &d = s->d;
  CK(cudaStreamSynchronize(s->stream));
  const int blocks = 8;
  const unsigned preset[4] = {(unsigned)blocks, 0u, 0u, 0u};     // arrivals already at the grid size
  const int zero[4] = {0, 0, 0, 0};
  TRY(h2d(s, d.gbar, preset, 4));
  TRY(h2d(s, d.err, zero, 4));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, s->stream));
  CK(pg_launch_barrier_probe(d, s->stream, blocks));
  CK(cudaEventRecord(e1, s->stream));
  CK(cudaEventSynchronize(e1));
  float ms = 0.0f;
  CK(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (wait_ms) *wait_ms = ms;
  int err[4];
  CK(cudaMemcpy(err, d.err, sizeof err, cudaMemcpyDeviceToHost));
  // leave the barrier and the error record clean for the session's own kernels
  const unsigned clean[4] = {0u, 0u, 0u, 0u};
  TRY(h2d(s, d.gbar, clean, 4));
  TRY(h2d(s, d.err, zero, 4));
  CK(cudaStreamSynchronize(s->stream));
  return err[0] == PG_ERR_TIMEOUT ? PG_OK : PG_ERR_ARGUMENT;
}

int pg_session_kernel_launches(pg_session *s, long long *count)
{
  if (!s || !count) return PG_ERR_ARGUMENT;
  *count = s->launches;
  return PG_OK;
}

} // extern "C"
