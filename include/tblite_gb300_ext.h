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
#include "tblite.h"
#ifdef __cplusplus
extern "C" {
#endif

/*
 * Batched single points.  No counterpart in the reference, which evaluates one molecule per
 * tblite_get_singlepoint call.  Energy and analytic gradient of nmol independent molecules:
 * mols[i] with calcs[i] (built by tblite_new_gfn2_calculator for that structure) into
 * results[i].  The molecules run through the SCF together, one launch per step for every size
 * bucket, each with its own calculator settings (accuracy, temperature, mixer damping and
 * memory, iteration limit) and its own convergence test; a result that already holds a
 * compatible wavefunction restarts that molecule, as in tblite_get_singlepoint.  A molecule
 * that the batch cannot finish (temperature annealing, more than the batch's Broyden history,
 * not converged, a failure) is evaluated by the one-molecule path afterwards, so every result
 * and error is what tblite_get_singlepoint gives.  Batched results hold energies, gradient,
 * virial, charges, multipoles, dipole, orbital energies and occupations; the density matrix
 * and orbital coefficients are not kept.  status[i] (may be NULL) is 0 on success and 1 when
 * molecule i failed; its message is pushed onto the context error log, prefixed with
 * "Batch entry i:".  Returns the number of failed molecules.
 */
int tblite_gb300_batch_singlepoint(tblite_context ctx, int nmol, const tblite_structure* mols,
                                   const tblite_calculator* calcs, const tblite_result* results,
                                   int* status);
/* molecules of the last batch call that took the one-molecule path */
int tblite_gb300_batch_last_fallbacks(void);
/* Density solver of the batched SCF for closed shells of at least 96 orbitals (the projection
 * threshold): 1 (default)
 * spectral projection (SP2 squarings on the tensor cores, P = 2 X D X^T; a molecule whose
 * HOMO-LUMO gap of the converged Fock matrix is below 80 kT, or whose projection does not
 * converge, is re-run by the one-molecule path), 0 diagonalisation for every molecule.  The
 * results are the same to the parity bar either way; orbital energies and occupations come
 * from a diagonalisation of the final Fock matrix. */
void tblite_gb300_set_batch_density_solver(int mode);
/* molecules of the last batch call whose SCF density came from the spectral projection */
int tblite_gb300_batch_last_projected(void);
/* density path of each molecule of the last batch call: 1 spectral projection, 0 batched
 * diagonalisation, -1 the one-molecule path; returns the number of molecules recorded */
int tblite_gb300_batch_last_modes(int* modes, int nmol);
/* Autotuner of the batch schedule: coordinate descent over CUDA graphs (kept, or switched off;
 * never switched on against tblite_gb300_set_batch_graphs), the projection threshold (64, 80, 96,
 * 112, 128, 144, 176 orbitals or off), the bucket cut (3/4, 2/3, 4/5 of the largest orbital count), the CTAs
 * per SM of the cluster tridiagonalisation (1, 2), the small-bucket tridiagonalisation (full
 * storage or packed) and the side streams (4, 8, 16), each candidate
 * timed as the wall time of a batch call (best of three) on a fixed pseudo-random sample of
 * `sample` of the given molecules (256 if <= 0); a candidate replaces the current choice only
 * when more than 1 % faster.  The fastest schedule stays set.  Returns the
 * number of timed calls, -1 if the sample could not be evaluated. */
int tblite_gb300_batch_autotune(tblite_context ctx, int nmol, const tblite_structure* mols,
                                const tblite_calculator* calcs, int sample);
/* the current batch schedule as text (written up to n - 1 characters); returns its length */
int tblite_gb300_batch_schedule(char* buf, int n);
/* back to the default batch schedule (CUDA graphs on) */
void tblite_gb300_batch_reset_schedule(void);
/* SCF iterations of a batch call as CUDA graphs (default 1): each iteration of a memory chunk
 * (every bucket on every side stream) is captured, instantiated once and updated in place while
 * its launch structure stays the same, and launched with one call.  Calls with the per-kernel
 * profiler enabled launch directly.  _last_graphs reports the instantiations and graph launches
 * of the last call (returns whether graphs are enabled). */
void tblite_gb300_set_batch_graphs(int enable);
int tblite_gb300_batch_last_graphs(int* builds, int* launches);
/* device time (ms, CUDA events) of the last batch call from the first setup kernel to the end
 * of the gradient, summed over its memory chunks (uploads, read-back and the one-molecule
 * path excluded) */
double tblite_gb300_batch_last_device_ms(void);
/* host wall time (ms) of the last batch call by phase, in this order: building the molecule
 * plans, chunking, staging and uploading the inputs, unpacking the results, the one-molecule
 * path, the whole call; fills up to n entries and returns the number of phases */
int tblite_gb300_batch_last_host_ms(double* ms, int n);
/* SCF iterations of each molecule of the last batch call; 0 for molecules routed to the
 * one-molecule path up front, a negative code for molecules that left the batch (-1 singular
 * Broyden system, -2 overlap not positive definite, -3 Fermi level above the eigenvalues the
 * batch computes, -4 iteration limit or Broyden history); returns the number of molecules */
int tblite_gb300_batch_last_iterations(int* iterations, int nmol);

/* batched GEMMs of molecules with at least 128 orbitals on the BF16 tensor cores with
 * FP64-accurate operand splitting (1, the default) or as FP64 tile GEMMs (0); process wide */
void tblite_gb300_set_split_gemm(int enable);
/* number of streams (1..16, default 8) over which a batch call spreads its size buckets; 1 runs
 * the buckets one after the other, so per-kernel event times bracket each kernel alone */
void tblite_gb300_set_batch_streams(int count);
/* smallest orbital count of a closed shell that takes the spectral projection in the batch (the
 * autotuner's threshold); a value <= 0 only queries.  Returns the previous value. */
int tblite_gb300_set_projection_threshold(int nao);
/* tridiagonalisation of batch buckets of at most 156 orbitals: 1 (default) the one-CTA kernel
 * with the full matrix in shared memory, 0 the packed lower-triangle kernel (a cluster of one or
 * two CTAs; two thirds of the FMAs) */
void tblite_gb300_set_small_tridiag(int full_storage);
/* schedule of the batched tridiagonalisation: 2 (default) clusters wide enough that two CTAs
 * share an SM (one computes while the other waits at a cluster barrier), 1 the narrowest
 * cluster whose CTAs fit the shared memory of one SM each */
void tblite_gb300_set_tridiag_ctas_per_sm(int count);

/* enable (1) or disable (0) event timing for subsequent single points (process wide) */
void tblite_gb300_set_profiling(int enable);

/* copy per-phase times (ms) and launch counts of the last single point; returns the number
 * of phases the library knows (9).  total_ms spans the first to the last recorded event. */
int tblite_gb300_get_profile(double* phase_ms, int* phase_count, int nphase, double* total_ms,
                             int* iterations);

/* per-kernel device times (ms, summed) and launch counts of the last single point, from CUDA
 * events around each launch on the engine stream (profiling enabled).  Slots: 0 Householder
 * tridiagonalisation, 1 eigenvalue multisection, 2 inverse iteration, 3 back-transformation,
 * 4 GEMM (all uses outside the pipelined split GEMM), 5 Fock assembly, 6 Mulliken column sums,
 * 7 pipelined split GEMM products of the batch (kb_opipe_sq, kb_opipe_site), 8 their operand
 * preparation (projection steps kb_sp2_step, exponents and slice images of the GEMM sites).
 * Returns the slot count. */
int tblite_gb300_get_kernel_profile(double* kernel_ms, int* kernel_count, int nslot);

/* channels of the bond orders tblite_get_result_bond_orders copies: 1 for a closed shell
 * (nat x nat), 2 for a restricted open shell (total and magnetisation, nat x nat x 2 in the
 * reference's column-major order), 0 when the result holds none (batched results) */
int tblite_gb300_get_result_bond_order_channels(tblite_result res);

/* Mulliken shell charges q_sh [nsh] of the last single point (the reference keeps them in its
 * wavefunction, wavefunction/type.f90 qsh, and writes them to restart files, but its C API has
 * no getter for them) */
void tblite_gb300_get_result_shell_charges(tblite_error error, tblite_result res, double* qsh);

/*
 * Shell parameters and the parameter gradient (no counterpart in the reference C API; the
 * reference fits parameters through its Fortran parameter records).  Arrays are per shell of
 * the calculator (tblite_get_calculator_shell_count): self energy se0 (Hartree), its
 * coordination-number shift kcn (e_s = se0_s - kcn_s CN_A), chemical hardness eta and
 * hardness derivative Gamma (third order).  NULL leaves an array untouched.
 * With the parameter gradient enabled, tblite_get_singlepoint also stores dE/d(parameter) of
 * the converged energy (explicit derivative at the final density, which the variational SCF
 * makes exact).
 */
void tblite_gb300_set_calculator_parameter_gradient(tblite_context ctx, tblite_calculator calc,
                                                    int enable);
void tblite_gb300_get_calculator_shell_parameters(tblite_context ctx, tblite_calculator calc,
                                                  double* selfenergy, double* kcn,
                                                  double* hubbard, double* hubbard_deriv);
void tblite_gb300_set_calculator_shell_parameters(tblite_context ctx, tblite_calculator calc,
                                                  const double* selfenergy, const double* kcn,
                                                  const double* hubbard,
                                                  const double* hubbard_deriv);
void tblite_gb300_get_result_parameter_gradient(tblite_error error, tblite_result res,
                                                double* dselfenergy, double* dkcn,
                                                double* dhubbard, double* dhubbard_deriv);
/* Slater exponent of every shell (calculator shell order); setting them redoes the STO-nG
 * expansion of each shell (GFN2-xTB calculators) */
void tblite_gb300_get_calculator_slater_exponents(tblite_context ctx, tblite_calculator calc,
                                                   double* zeta);
void tblite_gb300_set_calculator_slater_exponents(tblite_context ctx, tblite_calculator calc,
                                                   const double* zeta);
/* dE/d(Slater exponent) per shell, stored by a single point with the parameter gradient on */
void tblite_gb300_get_result_slater_gradient(tblite_error error, tblite_result res, double* dzeta);

/*
 * Density solver of the calculator's next single points.  0 (default): the reference's
 * diagonalisation (scf/diag.f90:62-143: generalised eigenproblem, Fermi filling,
 * P = C f C^T).  1: spectral projection for large gapped closed-shell systems: Loewdin
 * orthogonalisation by Newton-Schulz, second-order projection (SP2) of the orthogonalised
 * Fock matrix, P = 2 Z X Z and W = P F P / 2, all products on the tensor cores.  It fills the
 * reference's solver slot (scf/solver.f90:28-45, get_density / get_wdensity).  A single point
 * with solver 1 fails for open shells and for a HOMO-LUMO gap below 80 kT (certified by
 * Lanczos); its result has no orbital energies, occupations or coefficients.
 */
void tblite_gb300_set_calculator_density_solver(tblite_context ctx, tblite_calculator calc,
                                                int solver);
/* HOMO, LUMO (Hartree) and the bound on the sum of their errors, certified by solver 1 */
void tblite_gb300_get_result_gap(tblite_error error, tblite_result res, double* gap);

/*
 * C = A B on the pipelined FP64-accurate split GEMM (BF16 tensor cores), device pointers,
 * column-major: A m x k (leading dimension m), B k x n (leading dimension k), C m x n (leading
 * dimension m); sym != 0: C is symmetric (m == n), its lower tiles are computed and mirrored.
 * stream: a cudaStream_t (NULL: the default stream); the call synchronises it.  Returns 0, 1 if
 * the tensor-core pipeline did not answer within its wait limit, -1 on bad arguments, -2 on a
 * CUDA error.  No counterpart in the reference (its products are BLAS dgemm calls).
 */
int tblite_gb300_split_gemm(int m, int n, int k, const double* a, const double* b, double* c,
                            int sym, void* stream);
/* products of the spectral-projection solver: 1 (default) pipelined split GEMM from slice
 * images, 0 the per-tile split GEMM */
void tblite_gb300_set_pipelined_gemm(int enable);

/* number of engine kernels launched since the library was loaded (all threads) */
unsigned long long tblite_gb300_get_launch_count(void);
/* algorithmic FP64 work (flop) of the one-molecule path's tensor-core split GEMMs since the
 * library was loaded: 2 M N K per product, N (N + 1) K per symmetric product */
unsigned long long tblite_gb300_get_split_gemm_flops(void);

/*
 * Density matrix P = C diag(f) C^T that allocates no device memory.  No counterpart in the
 * reference: it is the engine's density step (scf/diag.f90 get_density_matrix) for callers
 * that cannot allocate device memory when they need it, because a pool allocator already
 * owns the device or because cudaMalloc/cudaFree would synchronise the device on a
 * latency-bound loop.
 *
 *   n       number of orbitals (rows of C and order of P)
 *   k       number of leading columns of C that enter (0 <= k <= n)
 *   C       device pointer, column-major [k][n]: C[m*n + r] = coefficient of AO r in orbital m
 *   f       device pointer, occupations [k]
 *   P       device pointer, output [n][n] (symmetric)
 *   stream  cudaStream_t to launch on (NULL: the legacy default stream)
 *
 * Returns 0 on success, -1 for an invalid argument, -2 when n*k exceeds
 * tblite_gb300_density_matrix_noalloc_max() (nothing is launched), -3 for a CUDA error.
 * The workspace is one fixed device array per device inside the library (2^19 doubles,
 * 4 MiB).  Every call looks up its address with the caller's device current; the first
 * call on a device can load the library's device code there, so make that first call before
 * starting any stream capture.  P is exactly symmetric.  Calls that may overlap in time on
 * one device (other streams or threads) race on the array and must be serialised.
 */
int tblite_gb300_density_matrix_noalloc(int n, int k, const double* C, const double* f, double* P,
                                        void* stream);
/* Test hooks of the failure paths (no GPU fault is caused by either):
 * tblite_gb300_set_calculator_fault(ctx, calc, 1) makes every overlap factorisation of the
 * calculator report a pivot that is not positive, as a singular overlap (coincident atoms)
 * does: the single point fails with the reference's "(sygvd) failed to solve eigenvalue
 * problem. info=<n+1>", a batch entry leaves the batch and fails the same way (0 clears it).
 * tblite_gb300_set_pipeline_wait_limit(polls) sets how often a pipeline wait of the
 * pipelined split GEMM polls before it aborts the tile (0: the default 2^22); a wait that runs
 * out sets the status word (projection single point: an error; batch: the molecule takes the
 * one-molecule path).  Returns 0, or -1 on a CUDA error. */
void tblite_gb300_set_calculator_fault(tblite_context ctx, tblite_calculator calc, int kind);
int tblite_gb300_set_pipeline_wait_limit(int polls);
/* FP64-equivalent flop (2 m n K per output tile that ran) of the batched spectral projection's
 * squarings on the tensor cores since library load, counted on the device */
unsigned long long tblite_gb300_get_pipe_batch_flops(void);
/* largest n*k the fixed workspace of tblite_gb300_density_matrix_noalloc holds */
int tblite_gb300_density_matrix_noalloc_max(void);

#ifdef __cplusplus
}
#endif
#endif
