/* CPU FP64 restatement of the SUS2-SH E / F / virial path -- TEST INFRASTRUCTURE ONLY.
 *
 * This is the oracle the GPU engine is checked against.  It is never linked into, loaded by or
 * called from the product path; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline use it.  It is pinned against the reference implementation through the committed
 * golden fixtures in tests/golden/ (reference embedded engine and trainer outputs).
 */
#ifndef SUS2_ORACLE_H
#define SUS2_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif
/* Loads a .sus2 model; returns NULL and writes a message into err on failure. */
void* orc_load(const char* path, char* err, int errlen);
void orc_free(void* model);
int orc_param_count(void* model);
int orc_get_params(void* model, double* out);
int orc_set_params(void* model, const double* in);
double orc_get_scaling(void* model);
int orc_set_scaling(void* model, double scaling);
/* One periodic frame: cell rows are lattice vectors.  Outputs energy, forces[3n], virial[6]
 * (xx, yy, zz, xy, xz, yz), site energies[n] (any may be NULL).  threads <= 0: all cores.
 * Returns the number of directed edges, or -1 on error (message in err). */
long long orc_efs(void* model, int n, const double* cell, const double* pos, const int* types, double* energy,
                  double* forces, double* virial, double* site, int threads, char* err, int errlen);
/* Same, also returning seconds[2] = {edge build, E/F/virial compute}. */
long long orc_efs_timed(void* model, int n, const double* cell, const double* pos, const int* types, double* energy,
                        double* forces, double* virial, double* site, int threads, double* seconds, char* err,
                        int errlen);
/* The periodic frame's directed edge set (strict r < cutoff, self images included, d = x_j - x_i),
 * in centre order (the image-scan rule of Neighborhoods::InitNbhs, src/neighborhoods.cpp:358):
 * writes at most cap edges (arrays may be NULL), returns the total or -1. */
long long orc_edges(void* model, int n, const double* cell, const double* pos, long long cap, int* ei, int* ej,
                    double* d, char* err, int errlen);
/* Caller edge list (single domain, owned centres 0..nowned-1 of nall atoms). */
int orc_efs_edges(void* model, int nowned, int nall, const int* types, int nedges, const int* ei, const int* ej,
                  const double* d, double* energy, double* forces, double* virial, double* site, char* err, int errlen);
/* Parameter gradient of  sum_i ew_i E_i + sum_i fw_i . F_i + sum_ab sw_ab S_ab  where F are forces and
 * S = -sum_e d (x) dE/dd the 3x3 virial; accumulates into grad[param_count].  Uses the image-scan
 * edges of one periodic frame.  Returns 0 or -1. */
int orc_grad(void* model, int n, const double* cell, const double* pos, const int* types, const double* ew,
             const double* fw, const double* sw, double* grad, char* err, int errlen);
/* orc_grad plus the Effect gate-x L2 term of the reference objective with coefficient gate_x:
 * *penalty = the term's value for this configuration, grad += its parameter gradient as well. */
/* Dimensions and parameter offsets: out[12] = {C, S, B, F, species_readout, o_shift, o_radial,
 * o_species, o_linear, nparams, nblk, K}. */
int orc_layout(void* model, int* out);
/* Per-atom descriptors (the S scalar moments, MLMTPR::CalcDescriptors) of one frame, desc[n][S]. */
int orc_descriptors(void* model, int n, const double* cell, const double* pos, const int* types, double* desc,
                    char* err, int errlen);
int orc_grad_gatex(void* model, int n, const double* cell, const double* pos, const int* types, const double* ew,
                   const double* fw, const double* sw, double gate_x, double* grad, double* penalty, char* err,
                   int errlen);
#ifdef __cplusplus
}
#endif
#endif
