/*
 * Extensions of libtblite_gb300.so beyond the tblite C API.
 *
 * Instrumentation: per-phase device times of the last tblite_get_singlepoint call,
 * measured with CUDA events on the engine's stream.  These entry points have no
 * counterpart in the reference (tblite 0.7.0); they exist for benchmarking.
 *
 * Phases: 0 setup (CN, integrals + H0, repulsion, Cholesky of S), 1 potentials,
 *         2 Fock assembly, 3 eigensolve, 4 Fermi filling + density matrix,
 *         5 Mulliken analysis + energies, 6 Broyden mixing, 7 nuclear gradient,
 *         8 device-to-host result transfer.
 */
#ifndef TBLITE_GB300_EXT_H
#define TBLITE_GB300_EXT_H
#ifdef __cplusplus
extern "C" {
#endif

/* enable (1) or disable (0) event timing for subsequent single points (process wide) */
void tblite_gb300_set_profiling(int enable);

/* copy per-phase times (ms) and launch counts of the last single point; returns the number
 * of phases the library knows (9).  total_ms spans the first to the last recorded event. */
int tblite_gb300_get_profile(double* phase_ms, int* phase_count, int nphase, double* total_ms,
                             int* iterations);

#ifdef __cplusplus
}
#endif
#endif
