// pg_meshcontact.h -- device state of the mesh-mesh contact stage
// (pg_meshcontact.cu): triangle boxes and cell sort, the pairs of this and
// the previous step, and the per-particle entry sort.
#pragma once
#include <cuda_runtime.h>
#include "pg_state.h"

#define PG_TT_KMAX 64             // partners one triangle may find (the search's thread-local list)

struct PgTT
{
  double r = 0.0;                 // swept radius of every mesh triangle
  double h = 0.0, org[3] = {0, 0, 0};
  int dim[3] = {1, 1, 1}, ncells = 1;
  unsigned none = 0, enone = 0;   // sentinel keys (above every cell / particle)
  int passes = 2, epasses = 2;    // radix-sort passes of the two sorts
  int kmax = PG_TT_KMAX;          // partners one triangle may find
  unsigned char *big = nullptr;   // [trinum] 1: larger than a cell
  // [trinum] box widened by r, as keys whose unsigned order is the IEEE
  // order of the coordinates (-0 = +0): min xyz (NaN: above every key),
  // max xyz (NaN: 0), so that a NaN fails every overlap test
  unsigned long long *box[6] = {};
  int *cell = nullptr;            // [trinum] grid cell of a small triangle's box centre
  unsigned *keys[2] = {}; int *vals[2] = {}; unsigned *hist = nullptr;
  int *cstart = nullptr, *cend = nullptr;   // [ncells + 1]: the last range holds the big triangles
  int *cand = nullptr;            // [kmax][trinum] partners found, sorted
  int *cnt = nullptr, *off = nullptr;       // [trinum], [trinum + 1]
  int *np_dev = nullptr;          // pairs of this step
  int cap = 0;                    // pair capacity
  int np_last = 0;                // pairs of the last step
  int *pf = nullptr, *pu = nullptr;         // [cap] finder and partner of each pair
  int *queue = nullptr, *qn = nullptr;      // [cap] pairs that are not plainly apart, their count
  unsigned char *act = nullptr;
  double *st[3] = {}, *f[3] = {}, *p[3] = {};   // tangential state, force on the finder's particle, point
  // the previous step's pairs (state carried by (finder, partner))
  int *poff = nullptr, *ppu = nullptr;
  unsigned char *pact = nullptr;
  double *pst[3] = {};
  unsigned *ekeys[2] = {}; int *evals[2] = {}; unsigned *ehist = nullptr;
  int *pfirst = nullptr, *plast = nullptr;  // [parnum] each particle's entries
  // sums in chunks of PG_TT_CHUNK entries: chunks per particle, their
  // offsets (an exclusive scan), the chunk sums (force, torque)
  int *nch = nullptr, *choff = nullptr, *nchunks = nullptr;
  double *csum[6] = {};
  long long ccap = 0;             // chunk-sum capacity
};

#define PG_TT_CHUNK 1024          // entries one warp sums into one chunk sum

int pg_tt_key_bits(int ncells);
void pg_tt_find(const PgDev &d, PgTT &g, cudaStream_t s);                 // steps 1-4a; total in g.np_dev
void pg_tt_forces(const PgDev &d, PgTT &g, cudaStream_t s, int np, double step);   // steps 4b-6
int pg_tt_kernel_count(const PgTT &g, int trinum, int np);
long long pg_tt_max_chunks(int parnum, int np);   // chunk sums a step can need
