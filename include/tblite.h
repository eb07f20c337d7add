/*
 * C API of the GB300 GFN2-xTB engine (libtblite_gb300.so).
 *
 * Drop-in replacement for the single-point subset of the tblite C API.  Every entry point
 * below has the same name, argument list and error convention as the reference header it
 * replaces (tblite 0.7.0, include/tblite/<file>.h:<line> cited per declaration):
 *
 *   - handles are opaque pointers owned by the caller and released with tblite_delete_*,
 *     which also sets the handle to NULL;
 *   - calls taking a tblite_error record failures there (tblite_check_error returns 1);
 *   - calls taking a tblite_context push failures onto the context error log
 *     (tblite_check_context returns 1, tblite_get_context_error pops the message);
 *   - units are Bohr, Hartree, Hartree/Bohr; electronic temperature in Hartree;
 *   - arrays are caller allocated, C row-major ([nat][3], [nao][nao], ...), which matches
 *     the Fortran column-major layout of the reference.
 *
 * All arithmetic runs in FP64 on the GPU (CUDA, sm_103a).  There is no CPU fallback: if
 * no CUDA device is usable the calls fail with an error message.
 */
#ifndef TBLITE_GB300_H
#define TBLITE_GB300_H

#ifdef __cplusplus
#include <cstdbool>
extern "C" {
#else
#include <stdbool.h>
#endif

#ifdef TBLITE_CFFI /* cffi parses the preprocessed header: plain declarations */
#define TBLITE_API_ENTRY
#define TBLITE_API_CALL
#endif
#ifndef TBLITE_API_ENTRY
#define TBLITE_API_ENTRY extern
#endif
#ifndef TBLITE_API_CALL
#define TBLITE_API_CALL
#endif

/* ---- version / features: include/tblite/version.h:28-31, features.h:24-32 ---- */
TBLITE_API_ENTRY int TBLITE_API_CALL tblite_get_version(void);
TBLITE_API_ENTRY int TBLITE_API_CALL tblite_get_feature(const char* flag);

/* ---- error handling: include/tblite/error.h:30-63 ---- */
typedef struct _tblite_error* tblite_error;
TBLITE_API_ENTRY tblite_error TBLITE_API_CALL tblite_new_error(void);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_delete_error(tblite_error* error);
TBLITE_API_ENTRY int TBLITE_API_CALL tblite_check_error(tblite_error error);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_clear_error(tblite_error error);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_error(tblite_error error, char* buffer,
                                                       const int* buffersize);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_set_error(tblite_error error, char* buffer,
                                                       const int* buffersize);

/* ---- calculation context: include/tblite/context.h:32-100 ---- */
typedef struct _tblite_context* tblite_context;
typedef void (*tblite_logger_callback)(tblite_error, char*, int, void*);
TBLITE_API_ENTRY tblite_context TBLITE_API_CALL tblite_new_context(void);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_delete_context(tblite_context* ctx);
TBLITE_API_ENTRY int TBLITE_API_CALL tblite_check_context(tblite_context ctx);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_context_error(tblite_context ctx, char* buffer,
                                                               const int* buffersize);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_set_context_logger(tblite_context ctx,
                                                                tblite_logger_callback callback,
                                                                void* userdata);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_set_context_color(tblite_context ctx, int color);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_set_context_verbosity(tblite_context ctx,
                                                                   int verbosity);

/* ---- molecular structure: include/tblite/structure.h:34-106 ---- */
typedef struct _tblite_structure* tblite_structure;
TBLITE_API_ENTRY tblite_structure TBLITE_API_CALL
tblite_new_structure(tblite_error error, const int natoms, const int* numbers,
                     const double* positions, const double* charge, const int* uhf,
                     const double* lattice, const bool* periodic);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_delete_structure(tblite_structure* mol);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_update_structure_geometry(tblite_error error,
                                                                      tblite_structure mol,
                                                                      const double* positions,
                                                                      const double* lattice);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_update_structure_charge(tblite_error error,
                                                                    tblite_structure mol,
                                                                    const double* charge);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_update_structure_uhf(tblite_error error,
                                                                 tblite_structure mol,
                                                                 const int* uhf);

/* ---- single point results: include/tblite/result.h:31-264 ---- */
typedef struct _tblite_result* tblite_result;
TBLITE_API_ENTRY tblite_result TBLITE_API_CALL tblite_new_result(void);
TBLITE_API_ENTRY tblite_result TBLITE_API_CALL tblite_copy_result(tblite_result res);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_delete_result(tblite_result* res);
/* Save / load the wavefunction of a result (NumPy .npz restart file with the reference's
 * member names; replaces include/tblite/result.h:253-265) */
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_save_result_wavefunction(tblite_error error,
                                                                      tblite_result res,
                                                                      const char* filename);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_load_result_wavefunction(tblite_error error,
                                                                      tblite_result res,
                                                                      const char* filename);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_result_number_of_atoms(tblite_error error,
                                                                       tblite_result res, int* nat);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_result_number_of_shells(tblite_error error,
                                                                        tblite_result res,
                                                                        int* nsh);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_result_number_of_orbitals(tblite_error error,
                                                                          tblite_result res,
                                                                          int* nao);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_result_number_of_spins(tblite_error error,
                                                                       tblite_result res,
                                                                       int* nspin);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_result_energy(tblite_error error,
                                                              tblite_result res, double* energy);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_result_energies(tblite_error error,
                                                                tblite_result res,
                                                                double* energies);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_result_gradient(tblite_error error,
                                                                tblite_result res,
                                                                double* gradient);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_result_virial(tblite_error error,
                                                              tblite_result res, double* sigma);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_result_charges(tblite_error error,
                                                               tblite_result res, double* charges);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_result_bond_orders(tblite_error error,
                                                                   tblite_result res, double* mbo);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_result_dipole(tblite_error error,
                                                              tblite_result res, double dipole[3]);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_result_quadrupole(tblite_error error,
                                                                  tblite_result res,
                                                                  double quadrupole[6]);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_result_orbital_energies(tblite_error error,
                                                                        tblite_result res,
                                                                        double* emo);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_result_orbital_occupations(tblite_error error,
                                                                           tblite_result res,
                                                                           double* occ);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_result_orbital_coefficients(tblite_error error,
                                                                            tblite_result res,
                                                                            double* cmat);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_result_density_matrix(tblite_error error,
                                                                      tblite_result res,
                                                                      double* pmat);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_result_overlap_matrix(tblite_error error,
                                                                      tblite_result res,
                                                                      double* smat);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_result_hamiltonian_matrix(tblite_error error,
                                                                          tblite_result res,
                                                                          double* hmat);

/* ---- calculator: include/tblite/calculator.h:36-291 ---- */
typedef enum {
  TBLITE_GUESS_SAD = 0,
  TBLITE_GUESS_EEQ = 1,
  TBLITE_GUESS_EEQBC = 2,
} tblite_guess;
typedef enum {
  TBLITE_MIXER_BROYDEN = 1,
} tblite_mixer;
typedef struct _tblite_calculator* tblite_calculator;
typedef struct {
  double smooth_cutoff;
} tblite_xtb_config;
TBLITE_API_ENTRY tblite_calculator TBLITE_API_CALL
tblite_new_gfn2_calculator(tblite_context ctx, tblite_structure mol, tblite_xtb_config* config);
/* GFN1-xTB parametrisation (calculator.h:79-82); elements whose GFN1 parameters carry a
   halogen-bond correction (Br, I, At) and d-shell elements are rejected */
TBLITE_API_ENTRY tblite_calculator TBLITE_API_CALL
tblite_new_gfn1_calculator(tblite_context ctx, tblite_structure mol, tblite_xtb_config* config);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_delete_calculator(tblite_calculator* calc);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_set_calculator_accuracy(tblite_context ctx,
                                                                    tblite_calculator calc,
                                                                    double acc);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_set_calculator_max_iter(tblite_context ctx,
                                                                    tblite_calculator calc,
                                                                    int max_iter);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_set_calculator_mixer_damping(tblite_context ctx,
                                                                         tblite_calculator calc,
                                                                         double damping);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_set_calculator_mixer_memory(tblite_context ctx,
                                                                        tblite_calculator calc,
                                                                        int memory);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_set_calculator_mixer(tblite_context ctx,
                                                                 tblite_calculator calc,
                                                                 tblite_mixer mixer);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_set_calculator_temperature_annealing(
    tblite_context ctx, tblite_calculator calc, double initial_etemp, int hold, int cycles);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_set_calculator_guess(tblite_context ctx,
                                                                 tblite_calculator calc,
                                                                 tblite_guess guess);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_set_calculator_temperature(tblite_context ctx,
                                                                       tblite_calculator calc,
                                                                       double etemp);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_set_calculator_save_integrals(tblite_context ctx,
                                                                          tblite_calculator calc,
                                                                          int save_integrals);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_calculator_shell_count(tblite_context ctx,
                                                                       tblite_calculator calc,
                                                                       int* nsh);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_calculator_shell_map(tblite_context ctx,
                                                                     tblite_calculator calc,
                                                                     int* sh2at);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_calculator_angular_momenta(tblite_context ctx,
                                                                           tblite_calculator calc,
                                                                           int* am);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_calculator_orbital_count(tblite_context ctx,
                                                                         tblite_calculator calc,
                                                                         int* nao);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_calculator_orbital_map(tblite_context ctx,
                                                                       tblite_calculator calc,
                                                                       int* ao2sh);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_singlepoint(tblite_context ctx,
                                                            tblite_structure mol,
                                                            tblite_calculator calc,
                                                            tblite_result res);

/* ---- interaction containers: include/tblite/container.h:31, 61-70 ---- */
typedef struct _tblite_container* tblite_container;
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_calculator_push_back(tblite_context ctx,
                                                                 tblite_calculator calc,
                                                                 tblite_container* cont);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_delete_container(tblite_container* cont);

/* ---- implicit solvation: include/tblite/solvation.h:30-52, 104-109 ----
 * Available here: ALPB with the GFN2 parameters (version tblite_solvation_alpb_gfn2) for the
 * solvent "water", with its CDS and free-energy shift terms; other solvents and models report
 * an error. */
enum tblite_ref_solvation_state {
  tblite_state_gsolv = 1,
  tblite_state_bar1mol = 2,
  tblite_state_reference = 3,
};
enum tblite_solvation_param {
  tblite_solvation_gbe = 10,
  tblite_solvation_alpb_gfn1 = 11,
  tblite_solvation_alpb_gfn2 = 12,
  tblite_solvation_gb = 20,
  tblite_solvation_gbsa_gfn1 = 21,
  tblite_solvation_gbsa_gfn2 = 22,
};
TBLITE_API_ENTRY tblite_container TBLITE_API_CALL
tblite_new_alpb_solvation_solvent(tblite_error error, tblite_structure mol, char* solvent,
                                  enum tblite_solvation_param version,
                                  enum tblite_ref_solvation_state refstate);

#ifdef __cplusplus
}
#endif

#endif /* TBLITE_GB300_H */
