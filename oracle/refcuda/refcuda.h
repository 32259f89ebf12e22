/* Host driver for the reference's own CUDA kernels (compiled from the
 * reference's sources into device-only cubins by oracle/refbuild, target
 * `cuda`). Test and baseline infrastructure: the product never loads it.
 * refcuda.cu says which reference host code each call restates. */
#ifndef REFCUDA_H
#define REFCUDA_H

#ifdef __cplusplus
extern "C" {
#endif

#define REFCUDA_OK 0
#define REFCUDA_ERR 1

typedef struct refcuda_solver refcuda_solver;

/* The message of the last failure. */
const char* refcuda_error(void);

/* A solver on the reference's cuda platform: equation euler1/2/3, flux
 * hll/hll3, reconstruction weno2, integrator forwardeuler/rungekutta2/
 * rungekutta3, boundary periodic/neumann. cubin_dir holds the five cubins. */
int refcuda_create(const char* cubin_dir, const char* equation, const char* flux, const char* reconstruction,
                   const char* integrator, const char* boundary, const int n[3], const double lower[3],
                   const double upper[3], double gamma, double cfl, refcuda_solver** out);
void refcuda_destroy(refcuda_solver* s);

/* The conserved state, padded, variable after variable (rho, m..., E), each
 * x fastest; set_state applies the boundary and resets time and counters. */
int refcuda_set_state(refcuda_solver* s, const double* host);
int refcuda_get_state(refcuda_solver* s, double* host);

/* Steps until t >= end_time or max_steps steps (max_steps <= 0: no limit);
 * number_of_saves > 0 adds the fixed-interval writer's dt clamp. */
int refcuda_run(refcuda_solver* s, double end_time, int number_of_saves, int max_steps, double* t_out,
                int* steps_out);

/* The demangled-name fragments of the kernels a configuration launches, one
 * per line, each matching exactly one kernel of the cubins. */
int refcuda_kernel_names(const char* equation, const char* flux, const char* boundary, char* out, int capacity);

/* Milliseconds of the last run (CUDA events on the legacy default stream
 * around the step loop), kernel launches so far, padded cells per variable. */
float refcuda_last_ms(const refcuda_solver* s);
long refcuda_launches(const refcuda_solver* s);
long refcuda_padded_cells(const refcuda_solver* s);

#ifdef __cplusplus
}
#endif
#endif
