/* Readers for the reference's run files: the inputs its command-line driver loads
 * from a path prefix (src/main.cpp:221-386, src/TUPSLoadingUtils.cpp:10-360).
 *
 *   <prefix>_Initial.dat         "bitstring,re[,im]" per line; bit i of the basis index is
 *                                the i-th character from the right; a bitstring alone has
 *                                coefficient 1; the qubit count is the longest bitstring
 *   <prefix>_Operators.dat       "a b c d" per operator, 1-based, 0 = absent
 *   <prefix>_Order.dat           "parameter" or "parameter,scale" per operator, 1-based
 *   <prefix>_Parameters.dat      angle sets: a count, a line with "= energy", the angles
 *                                (optional: without it there are no angle sets)
 *   <prefix>_Nuclear_Energy.dat  one number (optional)
 *   <prefix>_extractedmin        bare angle sets (read instead of the Parameters file's
 *                                sets when extracted_min is set)
 *
 * Angle sets are returned compressed, n_params angles each (n_params = largest order);
 * the angle of parameter p is the file's p-th angle when the file's last set has more
 * than p angles (src/TUPSLoadingUtils.cpp:275-280), else 0.  n_unique is the reference
 * driver's own parameter count, max(n_params, angles in the file's last set), which
 * also sizes the sets of an extractedmin file (src/TUPSLoadingUtils.cpp:255, 287).
 *
 * Replaces: readCsvState (src/TUPSLoadingUtils.h:12-13), loadPath (:18-19),
 * loadParameters (:21-31), loadExtractedMin (:36-40), LoadNuclearEnergy (:16).
 * A manager-level one-call setup from the same files is setRunFiles in
 * AnsatzSynthInterface.h.
 *
 * Return codes: 0 ok, 2 bad arguments, 3 a required file is missing or malformed (the
 * message is in aegpu_run_files_error, per calling thread).  No GPU is used. */
#ifndef AEGPU_RUNFILES_H
#define AEGPU_RUNFILES_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct aegpu_run_files aegpu_run_files;

int aegpu_run_files_load(const char *prefix, int extracted_min, aegpu_run_files **out);
/* One file alone: AEGPU_RUN_FILE_INITIAL (an Initial file), AEGPU_RUN_FILE_OPERATORS (an
 * Operators file) or AEGPU_RUN_FILE_NUCLEAR (path is the prefix of a _Nuclear_Energy.dat
 * file; a missing file is not an error, nuclear then reads NaN); the other fields stay
 * empty. */
enum { AEGPU_RUN_FILE_INITIAL = 1, AEGPU_RUN_FILE_OPERATORS = 2, AEGPU_RUN_FILE_NUCLEAR = 3 };
int aegpu_run_file_read(const char *path, int kind, aegpu_run_files **out);
/* An order file for n_ops operators and a Parameters file (optional): orders, parameter
 * counts, angle sets and energies (loadParameters, src/TUPSLoadingUtils.cpp:176-296). */
int aegpu_run_files_parameters(const char *order_path, const char *parameter_path, int n_ops, aegpu_run_files **out);
const char *aegpu_run_files_error(void);
/* Any output pointer may be null.  n_ops counts the operators or, for a handle from
 * aegpu_run_files_parameters, the order relations. */
int aegpu_run_files_sizes(const aegpu_run_files *f, int *nq, int *n_initial, int *n_ops, int *n_params,
                          int *n_unique, int *n_sets);
/* initial_index[n_initial] (0-based, full 2^nq space); initial_coeff[2*n_initial]
 * (re, im interleaved); operators_1b[4*n_ops] (row per operator, 0 = absent);
 * order_1b[n_ops]; scale[n_ops]; sets[n_sets*n_params] (row per set); energies[n_sets]
 * (NaN where a set has none); nuclear: NaN when the file is missing.  Any output
 * pointer may be null. */
int aegpu_run_files_get(const aegpu_run_files *f, int *initial_index, double *initial_coeff, int *operators_1b,
                        int *order_1b, double *scale, double *sets, double *energies, double *nuclear);
void aegpu_run_files_free(aegpu_run_files *f);

#ifdef __cplusplus
}
#endif
#endif
