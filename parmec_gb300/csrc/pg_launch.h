// pg_launch.h -- host-side launchers of the device kernels.
#pragma once
#include <cuda_runtime.h>
#include <vector>
#include "pg_state.h"

// pg_step.cu
void pg_launch_invert(const PgDev &d, cudaStream_t s);
void pg_launch_iso_flags(const PgDev &d, cudaStream_t s, int p0, int p1);   // isotropic-inertia flags
void pg_launch_euler(const PgDev &d, cudaStream_t s, double step);
void pg_launch_shapes(const PgDev &d, cudaStream_t s, bool skip_analytical);
void pg_launch_obstacles_state(const PgDev &d, cudaStream_t s, double step);   // velocities from obsang/obslin
void pg_launch_contacts(const PgDev &d, cudaStream_t s, double step);
int pg_contacts_kernel_count(const PgDev &d);   // launches of one contact evaluation (either form)
void pg_launch_springs(const PgDev &d, cudaStream_t s, double step);
void pg_launch_spring_runs(const PgDev &d, cudaStream_t s);     // sums of the long flush runs
void pg_launch_unspring(const PgDev &d, cudaStream_t s);        // UNSPRING rules, after the springs
void pg_launch_torsion(const PgDev &d, cudaStream_t s, double step);   // torsion springs, before the force sums
void pg_launch_gather(const double *const *cols, int ncols, const int *idx, int n, double *out, cudaStream_t s);
void pg_launch_integrate(const PgDev &d, cudaStream_t s, double step);
void pg_launch_force_sums(const PgDev &d, cudaStream_t s);                          // forces() tail
void pg_launch_dynamics(const PgDev &d, cudaStream_t s, double step0, double step1); // dynamics()
// adaptive stepping (d.hs set): force sums with the stiffness terms, the step
// choice on the device (adaptive_timestep), and the rest of the step
void pg_launch_force_sums_adapt(const PgDev &d, cudaStream_t s);
void pg_launch_adapt_step(const PgDev &d, cudaStream_t s);
void pg_launch_dynamics_fused(const PgDev &d, cudaStream_t s);
void pg_launch_critical_perspring(const PgDev &d, cudaStream_t s, double *h, double *om, double *ra);
void pg_launch_critical_perparticle(const PgDev &d, cudaStream_t s, double *ke, int use_contacts, double *h,
                                    double *om, double *ra);
void pg_launch_eqm_one(const PgDev &d, cudaStream_t s, int part2, const double *pts, double *out);
void pg_launch_restrain_velocities(const PgDev &d, cudaStream_t s);   // once per DEM call
void pg_launch_restrain_forces(const PgDev &d, cudaStream_t s);       // drop-in export (fused steps do it in k_integrate)
void pg_launch_mesh(const PgDev &d, cudaStream_t s);
void pg_launch_obstacles_row(const PgDev &d, cudaStream_t s, double step);     // velocities from the step table
void pg_launch_tail(const PgDev &d, cudaStream_t s, double step);
void pg_launch_obstacles_tail(const PgDev &d, cudaStream_t s, double step);  // both, one launch when it can
int pg_obstacles_kernel_count(const PgDev &d);
void pg_launch_excite(const PgDev &d, cudaStream_t s, double step);
int  pg_step_kernel_count(const PgDev &d);

// pg_mixed.cu
void pg_launch_mx_from64(const PgDev &d, cudaStream_t s, int p0 = 0, int p1 = -1, int e0 = 0, int e1 = -1);
void pg_launch_mx_inertia(const PgDev &d, cudaStream_t s);
void pg_launch_mx_to64(const PgDev &d, cudaStream_t s, int p0 = 0, int p1 = -1);
void pg_launch_mx_centres(const PgDev &d, cudaStream_t s);   // before a due rebuild
void pg_launch_contacts_mx(const PgDev &d, cudaStream_t s, double step);
void pg_launch_integrate_mx(const PgDev &d, cudaStream_t s, double step);
// the persistent fused step of the mixed form: shape index into the kernel
// table, threads per block and blocks of the cooperative grid
struct PgFusedCfg { int shape, threads, blocks; };
int  pg_fused_candidates(PgFusedCfg *out, int cap);
cudaError_t pg_launch_fused_mx(const PgDev &d, cudaStream_t s, double step, int nsteps, const PgFusedCfg &c);

// pg_session.cu
// spring flush runs longer than this are summed by k_spring_runs
#define PG_SPRING_RUN_LONG 64
void pg_spring_events(int P, int S, const int *sj, const int *sk, std::vector<int> &first, std::vector<int4> &ev,
                      std::vector<int4> &big);

// pg_sort.cu
int  pg_sort_blocks(int n);
// histogram scratch a radix sort of n keys needs (pg_launch_radix_sort):
// 256 counts per tile, and past PG_SORT_SCAN_ONE_BLOCK tiles the sums of the
// scan's tiles after them
#define PG_SORT_SCAN_ONE_BLOCK 32
size_t pg_sort_hist_len(int n);
int  pg_sort_kernel_count(int n, int passes);   // kernels one radix sort launches
int  pg_sort_passes(int bits_per_axis);
int  pg_sort_passes_bits(int key_bits);
void pg_launch_cell_keys(const double *x, const double *y, const double *z, int n, const double org[3],
                         double cell, const int dim[3], unsigned *keys, int *vals,
                         double *rx, double *ry, double *rz, const int *gate, cudaStream_t s,
                         const int *scene = nullptr, double *const sorg[3] = nullptr, int shift = 0);
void pg_launch_radix_sort(unsigned *k0, int *v0, unsigned *k1, int *v1, unsigned *hist, int n, int passes,
                          const int *gate, cudaStream_t s);
int  pg_scan_blocks(int n);                                   // scan block sums for n elements
int  pg_sort_passes_exact(int key_bits);                      // 8-bit passes, not rounded to even

// pg_rebuild.cu
void pg_launch_rebuild(const PgDev &d, cudaStream_t s);
cudaError_t pg_launch_barrier_probe(const PgDev &d, cudaStream_t s, int blocks);   // see pg_session_barrier_selftest
void pg_launch_rebuild_gate(const PgDev &d, cudaStream_t s);   // sets *rebuild when a sphere or vertex moved
int  pg_rebuild_kernel_count(const PgDev &d);
void pg_rebuild_grid_params(PgDev &d, const double *ext, double rmax, double rmin);
void pg_rebuild_key_bits(PgDev &d);
int  pg_rebuild_sort_bits(const PgDev &d);
int  pg_rebuild_entry_bits(int parnum);                         // key bits of the slave-entry sort
