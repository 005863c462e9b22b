/* parmec_coupling.h -- the library interface of parmec (parmec.h:291-310)
 * for C and C++ callers, over the GB300 DEM session.
 *
 * libparmec_gb300_coupling.so embeds the Python interpreter (or joins the
 * one of the calling process) and drives the package's commands, as the
 * reference's libparmec8 drives its own: decks are read by
 * pg_parmec_input, DEM runs on the GPU, and coupling codes exchange body
 * forces with it between DEM calls.  Every function returns 0 (or a
 * non-negative value) on success and -1 after printing the Python error.
 * Calls must come from one thread at a time. */
#ifndef PARMEC_COUPLING_H
#define PARMEC_COUPLING_H

#ifdef __cplusplus
extern "C" {
#endif

/* parmec::init (parmec.cpp:2227): empty buffers, reset the model */
int pg_parmec_init(void);

/* parmec::reset (parmec.cpp:2253) */
int pg_parmec_reset(void);

/* parmec::input (parmec.h:300): run the input deck at 'path' with its
 * ARGV() arguments argv[0..argc) */
int pg_parmec_input(const char *path, char **argv, int argc);

/* parmec::dem (parmec.h:303-310) without the interval callbacks and TSERIES
 * (decks set those): interval NULL or {files, history}, prefix NULL or the
 * output prefix; returns the run's wall time in seconds, or -1 */
double pg_parmec_dem(double duration, double step, const double *interval, const char *prefix, int verbose,
                     double adaptive);

/* declare_analytical (parmec.h:291): particle k's shapes leave contact
 * detection and the shape updates */
int pg_parmec_declare_analytical(int k);

/* prescribed_body_forces (parmec.h:281-289): the outer force and torque
 * added to particle k at every step of the next DEM calls (outer_force NULL
 * removes the entry), and the inner force and torque the particle had at
 * the last step before that addition */
int pg_parmec_set_body_force(int k, const double outer_force[3], const double outer_torque[3]);
int pg_parmec_get_body_force(int k, double inner_force[3], double inner_torque[3]);

/* particle count, and the position, linear and spatial angular velocity of particle k */
int pg_parmec_parnum(void);
int pg_parmec_particle(int k, double position[3], double linear[3], double angular[3]);

#ifdef __cplusplus
}
#endif

#endif
