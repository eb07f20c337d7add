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
#include <cstdint>
extern "C" {
#elif !defined(TBLITE_CFFI) /* cffi knows bool and int64_t itself: no system headers */
#include <stdbool.h>
#include <stdint.h>
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
#ifdef TBLITE_CFFI /* the callback the reference's Python package defines (context.h:42-45) */
extern "Python" void TBLITE_API_CALL logger_callback(tblite_error error, char* msg, int len,
                                                     void* user_data);
#endif
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

/* ---- post-processing dictionary: include/tblite/double_dictionary.h:28-110, result.h:243-246
 * A snapshot of a result's post-processing arrays ("bond-orders" [nat][nat][channels],
 * "molecular-dipole" [3], "molecular-quadrupole" [6]); indices are 1-based as in the
 * reference; arrays come out in Fortran order, unused trailing dimensions reported as 0. */
typedef struct _tblite_double_dictionary* tblite_double_dictionary;
TBLITE_API_ENTRY tblite_double_dictionary TBLITE_API_CALL
tblite_get_post_processing_dict(tblite_error error, tblite_result res);
TBLITE_API_ENTRY int TBLITE_API_CALL tblite_get_n_entries_dict(tblite_error error,
                                                              tblite_double_dictionary dict);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_array_entry_index(tblite_error error,
                                                                  tblite_double_dictionary dict,
                                                                  const int* index, double* array);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_array_size_index(tblite_error error,
                                                                 tblite_double_dictionary dict,
                                                                 const int* index, int* dim1,
                                                                 int* dim2, int* dim3);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_array_entry_label(tblite_error error,
                                                                  tblite_double_dictionary dict,
                                                                  char* label, double* array);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_array_size_label(tblite_error error,
                                                                 tblite_double_dictionary dict,
                                                                 char* label, int* dim1,
                                                                 int* dim2, int* dim3);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_get_label_entry_index(tblite_error error,
                                                                  tblite_double_dictionary dict,
                                                                  const int* index, char* label,
                                                                  const int* buffersize);
TBLITE_API_ENTRY void TBLITE_API_CALL
tblite_delete_double_dictionary(tblite_double_dictionary* dict);

/* ---- data tables: include/tblite/table.h:26-316 ----
 * Nested key/value tables (booleans, 64-bit integers, doubles, strings, arrays of those,
 * sub-tables), e.g. parameter sets in the reference's TOML layout.  Handles returned by
 * add_table / get_table / get_array refer to the parent's entry and stay valid on their own;
 * every handle is released with its delete call.  Array and key indices are 1-based. */
typedef struct _tblite_table* tblite_table;
typedef struct _tblite_array* tblite_array;
enum tblite_table_value_type {
  TBLITE_TABLE_VALUE_TYPE_NONE = 0,
  TBLITE_TABLE_VALUE_TYPE_BOOL = 1,
  TBLITE_TABLE_VALUE_TYPE_INT = 2,
  TBLITE_TABLE_VALUE_TYPE_DOUBLE = 3,
  TBLITE_TABLE_VALUE_TYPE_CHAR = 4,
  TBLITE_TABLE_VALUE_TYPE_ARRAY = 5,
  TBLITE_TABLE_VALUE_TYPE_TABLE = 6
};
TBLITE_API_ENTRY tblite_table TBLITE_API_CALL tblite_new_table(tblite_table* table);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_delete_table(tblite_table* table);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_table_set_double(tblite_error error,
                                                             tblite_table table, char key[],
                                                             double* value, int n);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_table_set_int64_t(tblite_error error,
                                                              tblite_table table, char key[],
                                                              int64_t* value, int n);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_table_set_bool(tblite_error error, tblite_table table,
                                                           char key[], bool* value, int n);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_table_set_char(tblite_error error, tblite_table table,
                                                           char key[], char (*value)[], int n);
TBLITE_API_ENTRY tblite_table TBLITE_API_CALL tblite_table_add_table(tblite_error error,
                                                                    tblite_table table,
                                                                    char key[]);
TBLITE_API_ENTRY tblite_array TBLITE_API_CALL tblite_new_array(void);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_delete_array(tblite_array* array);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_array_push_back_double(tblite_error error,
                                                                   tblite_array array,
                                                                   double value);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_array_push_back_int64_t(tblite_error error,
                                                                    tblite_array array,
                                                                    int64_t value);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_array_push_back_bool(tblite_error error,
                                                                 tblite_array array, bool value);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_array_push_back_char(tblite_error error,
                                                                 tblite_array array,
                                                                 char value[]);
TBLITE_API_ENTRY int TBLITE_API_CALL tblite_array_size(tblite_error error, tblite_array array);
TBLITE_API_ENTRY int TBLITE_API_CALL tblite_array_get_type(tblite_error error, tblite_array array,
                                                          int index);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_array_get_double(tblite_error error,
                                                             tblite_array array, int index,
                                                             double* value);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_array_get_int64_t(tblite_error error,
                                                              tblite_array array, int index,
                                                              int64_t* value);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_array_get_bool(tblite_error error, tblite_array array,
                                                           int index, bool* value);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_array_get_char(tblite_error error, tblite_array array,
                                                           int index, char value[], int n);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_table_set_array(tblite_error error,
                                                            tblite_table table, char key[],
                                                            tblite_array array);
TBLITE_API_ENTRY int TBLITE_API_CALL tblite_table_get_type(tblite_error error, tblite_table table,
                                                          char key[]);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_table_get_bool(tblite_error error, tblite_table table,
                                                           char key[], bool* value);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_table_get_int64_t(tblite_error error,
                                                              tblite_table table, char key[],
                                                              int64_t* value);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_table_get_double(tblite_error error,
                                                             tblite_table table, char key[],
                                                             double* value);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_table_get_char(tblite_error error, tblite_table table,
                                                           char key[], char value[], int n);
TBLITE_API_ENTRY tblite_table TBLITE_API_CALL tblite_table_get_table(tblite_error error,
                                                                    tblite_table table,
                                                                    char key[]);
TBLITE_API_ENTRY tblite_array TBLITE_API_CALL tblite_table_get_array(tblite_error error,
                                                                    tblite_table table,
                                                                    char key[]);
TBLITE_API_ENTRY int TBLITE_API_CALL tblite_table_get_n_keys(tblite_error error,
                                                            tblite_table table);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_table_get_key(tblite_error error, tblite_table table,
                                                          int index, char key[], int n);
/* write the table as TOML text to a file */
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_dump_table(tblite_error error, tblite_table table,
                                                       char filename[]);

/* ---- parametrisation records: include/tblite/param.h:26-80 ----
 * The global constants and element records of an xTB method.  export_* fill a record with a
 * built-in method's parameters; load / dump read and write it as a data table in the
 * reference's TOML layout (levels and CN shifts in eV there); tblite_new_xtb_calculator makes
 * a calculator from it (the GFN2-xTB form, or the GFN1-xTB form to which IPEA1-xTB belongs). */
typedef struct _tblite_param* tblite_param;
TBLITE_API_ENTRY tblite_param TBLITE_API_CALL tblite_new_param(void);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_delete_param(tblite_param* param);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_load_param(tblite_error error, tblite_param param,
                                                       tblite_table table);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_dump_param(tblite_error error, tblite_param param,
                                                       tblite_table table);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_export_gfn2_param(tblite_error error,
                                                              tblite_param param);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_export_gfn1_param(tblite_error error,
                                                              tblite_param param);
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_export_ipea1_param(tblite_error error,
                                                               tblite_param param);

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
/* calculator from a parametrisation record (calculator.h:92-107).  The GFN2-xTB form (CN
 * "dexp", self-consistent D4, arithmetic hardness average, shell-resolved third order, damped
 * multipoles) and the GFN1-xTB form (CN "exp", D3, harmonic average, atom-resolved third order,
 * its own element-pair factors) are available, with any element records and global constants;
 * other forms, d shells and the halogen-bond correction are refused with an error. */
TBLITE_API_ENTRY tblite_calculator TBLITE_API_CALL
tblite_new_xtb_calculator(tblite_context ctx, tblite_structure mol, tblite_param param,
                          tblite_xtb_config* config);
/* IPEA1-xTB (calculator.h:84-89): the GFN1 form with IPEA1-xTB's parameters */
TBLITE_API_ENTRY tblite_calculator TBLITE_API_CALL
tblite_new_ipea1_calculator(tblite_context ctx, tblite_structure mol, tblite_xtb_config* config);
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
/* post-processing of every single point (calculator.h:270-279): "bond-orders" or "molmom"
 * (molecular dipole and quadrupole), in the order added; without any, the first single point
 * adds both (the reference's default).  "xtbml" descriptors and TOML files report an error. */
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_push_back_post_processing_str(tblite_context ctx,
                                                                          tblite_calculator calc,
                                                                          tblite_structure mol,
                                                                          char* charptr);
/* post-processing from a parametrisation record (calculator.h:281-291): the records here carry
 * none, so this reports an error */
TBLITE_API_ENTRY void TBLITE_API_CALL tblite_push_back_post_processing_param(
    tblite_context ctx, tblite_calculator calc, tblite_structure mol, tblite_param param);

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
  tblite_solvation_ddcosmo = 100,
  tblite_solvation_ddcpcm = 101,
  tblite_solvation_ddpcm = 200
};
TBLITE_API_ENTRY tblite_container TBLITE_API_CALL
tblite_new_alpb_solvation_solvent(tblite_error error, tblite_structure mol, char* solvent,
                                  enum tblite_solvation_param version,
                                  enum tblite_ref_solvation_state refstate);
/* Further interactions (container.h:36-45, solvation.h:54-95): the homogeneous electric
 * field (three components, atomic units; NULL for a NULL argument; pushed into a GFN2-form
 * calculator), generalized Born with a dielectric constant (version 10 GB-epsilon with the ALPB
 * shape term or 20, Born kernel Still or P16); spin polarisation and ddX are not provided and
 * report an error. */
enum tblite_born_kernel {
  tblite_born_still = 1,
  tblite_born_p16 = 2,
};
TBLITE_API_ENTRY tblite_container TBLITE_API_CALL tblite_new_electric_field(double* efield);
TBLITE_API_ENTRY tblite_container TBLITE_API_CALL
tblite_new_spin_polarization(tblite_context ctx, tblite_structure mol, tblite_calculator calc,
                             double wscale);
TBLITE_API_ENTRY tblite_container TBLITE_API_CALL
tblite_new_gb_solvation_epsilon(tblite_error error, tblite_structure mol, double eps,
                                enum tblite_solvation_param version, enum tblite_born_kernel born);
TBLITE_API_ENTRY tblite_container TBLITE_API_CALL
tblite_new_ddx_solvation_epsilon(tblite_error error, tblite_structure mol, double eps,
                                 enum tblite_solvation_param model);
TBLITE_API_ENTRY tblite_container TBLITE_API_CALL
tblite_new_ddx_solvation_solvent(tblite_error error, tblite_structure mol, char* solvent,
                                 enum tblite_solvation_param model);

#ifdef __cplusplus
}
#endif

#if !defined(__cplusplus) && !defined(TBLITE_CFFI)
/* Generic macro to free an object handle (include/tblite.h:45-58) */
#define tblite_delete(ptr) _Generic((ptr), \
                       tblite_error: tblite_delete_error, \
                   tblite_container: tblite_delete_container, \
                     tblite_context: tblite_delete_context, \
                   tblite_structure: tblite_delete_structure, \
           tblite_double_dictionary: tblite_delete_double_dictionary, \
                  tblite_calculator: tblite_delete_calculator, \
                      tblite_result: tblite_delete_result, \
                       tblite_table: tblite_delete_table, \
                       tblite_param: tblite_delete_param \
                                   )(&ptr)
/* Generic macro to check for error status (include/tblite.h:60-67) */
#define tblite_check(ptr) _Generic((ptr), \
                      tblite_error: tblite_check_error, \
                    tblite_context: tblite_check_context \
                                  )(ptr)
#endif

#endif /* TBLITE_GB300_H */
