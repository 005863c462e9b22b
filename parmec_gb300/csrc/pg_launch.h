// pg_launch.h -- host-side launchers of the device kernels.
#pragma once
#include <cuda_runtime.h>
#include "pg_state.h"

// pg_step.cu
void pg_launch_invert(const PgDev &d, cudaStream_t s);
void pg_launch_euler(const PgDev &d, cudaStream_t s, double step);
void pg_launch_shapes(const PgDev &d, cudaStream_t s, bool skip_analytical);
void pg_launch_obstacles_state(const PgDev &d, cudaStream_t s, double step);   // velocities from obsang/obslin
void pg_launch_contacts(const PgDev &d, cudaStream_t s, double step);
void pg_launch_springs(const PgDev &d, cudaStream_t s, double step);
void pg_launch_integrate(const PgDev &d, cudaStream_t s, double step);
void pg_launch_mesh(const PgDev &d, cudaStream_t s);
void pg_launch_obstacles_row(const PgDev &d, cudaStream_t s, double step);     // velocities from the step table
void pg_launch_tail(const PgDev &d, cudaStream_t s, double step);
int  pg_step_kernel_count(const PgDev &d);

// pg_rebuild.cu
void pg_launch_rebuild(const PgDev &d, cudaStream_t s);
int  pg_rebuild_kernel_count(const PgDev &d);
void pg_rebuild_grid_params(PgDev &d, const double *lo, const double *hi, double rmax, double rmin);
