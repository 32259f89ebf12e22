/* CPU oracle for the alsfvm explicit finite-volume step and the alsuq
 * mean/variance statistics: a plain-C restatement of the reference's CPU
 * implementation.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE. Only the tests, the smoke check and
 * the CPU-baseline leg of the benchmark load this library, and only as the
 * checker. The product path (alsvinn_gb300/) never links or calls it.
 *
 * State layout matches the reference Volume: one padded array per conserved
 * variable, x fastest, (nx+2g)(ny+2g)(nz+2g) doubles, ghosts only in active
 * dimensions (alsfvm/src/volume/Volume.cpp:44-60, alsfvm/include/alsfvm/memory/
 * View.hpp:116-118); nvar arrays are stored back to back.
 *
 * Names are passed as the reference spells them in its XML configuration:
 * equation "euler1|euler2|euler3|burgers", flux "hll|hll3|godunov",
 * reconstruction "none|weno2|eno2|eno3|eno4", integrator
 * "forwardeuler|rungekutta2|rungekutta3", boundary "neumann|periodic".
 * Every function returns 0 on success and a negative code on error; the text
 * is available from fv_last_error(). */
#ifndef FVORACLE_H
#define FVORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

const char* fv_last_error(void);
void fv_set_threads(int n);
int fv_get_threads(void);

/* Ghost cells the reference allocates: max(flux stencil - 1, reconstruction
 * ghosts) (alsfvm/src/numflux/NumericalFluxCPU.cpp:226-231). */
int fv_ghost_cells(const char* recon);

int fv_boundary(const char* boundary, const int n[3], int ghosts, int nvar, double* U);

int fv_reconstruct(const char* equation, const char* recon, const int n[3], double gamma,
                   int direction, const double* U, double* left, double* right);

int fv_compute_flux(const char* equation, const char* flux, const char* recon, const int n[3],
                    double gamma, const double* U, double* out, double ws[3]);

int fv_run(const char* equation, const char* flux, const char* recon, const char* integrator,
           const char* boundary, const int n[3], const double lower[3], const double upper[3],
           double gamma, double cfl, double end_time, int number_of_saves, int max_steps,
           const double* prim, double* out, double* t_out, int* steps_out, double* dts,
           int max_dts);

/* Seconds the last fv_run on this thread spent in its step loop. */
double fv_last_loop_seconds(void);

int fv_prim_to_cons(const char* equation, const int n[3], int ghosts, double gamma,
                    const double* prim, double* cons);

int fv_obeys_constraints(const char* equation, const int n[3], int ghosts, double gamma,
                         const double* U);

int fv_uniform(int dimension, int sample, double lower, double upper, double* out);
int fv_generate_sequence(int nparams, const int* dims, const double* lowers, const double* uppers,
                         long long sample_start, long long nsamples, double* out);

int fv_structure_cube(const char* equation, const char* boundary, const int n[3], int ghosts, int number_of_h,
                      double p, const double* U, double* out);
int fv_meanvar(long count, int nsamples, const double* const* samples, double* mean,
               double* var);
int fv_structure_basic(const char* equation, const char* boundary, const int n[3], int ghosts, int number_of_h,
                       double p, int direction, const double* U, double* out);

/* Functionals of one padded state: identity, moment, legendre_pointwise,
 * log_entropy, bv, bv_direction, structure_cube. out (nvar x output cells,
 * x fastest) receives weight times the functional added to what it holds
 * (structure_cube overwrites and ignores the weight, as the reference does);
 * size_out receives the output extents. variable_mask selects the variables
 * of legendre_pointwise (bit k: variable k; 0: all). */
int fv_functional(const char* name, const char* equation, const char* boundary, const int n[3], int ghosts,
                  const double lower[3], const double upper[3], int degree, double min_value, double max_value,
                  unsigned variable_mask, double gamma, double p, int number_of_h, int direction, double weight,
                  const double* U, double* out, int size_out[3]);

#ifdef __cplusplus
}
#endif
#endif
