/* CPU oracle for the statevector hot path (test infrastructure only).
 * Restates pyquafu qfvm src/qfvm/statevector.hpp and simulator.hpp in C. */
#ifndef QSV_ORACLE_H
#define QSV_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Named-gate codes: the OPMAP table of src/qfvm/qasm.hpp:43-46 (same numbering
 * as QFVM_OP_* in include/qfvm_gb300.h). */
enum {
    QOR_X = 1, QOR_Y, QOR_Z, QOR_H, QOR_S, QOR_SDG, QOR_T, QOR_TDG, QOR_P,
    QOR_RX, QOR_RY, QOR_RZ, QOR_CX, QOR_CZ, QOR_CP, QOR_CCX, QOR_RZZ
};

void qor_one_targe_general(double* data, uint64_t size, const int32_t* posv, int npos, int ctrl_num, const double* mat);
void qor_one_targe_x(double* data, uint64_t size, const int32_t* posv, int npos, int ctrl_num);
void qor_one_targe_real(double* data, uint64_t size, const int32_t* posv, int npos, int ctrl_num, const double* mat);
void qor_one_targe_diag(double* data, uint64_t size, const int32_t* posv, int npos, int ctrl_num, const double* mat);
void qor_apply_x(double* data, uint64_t size, int32_t pos);
void qor_apply_y(double* data, uint64_t size, int32_t pos);
void qor_apply_z(double* data, uint64_t size, int32_t pos);
void qor_multi_targe_general(double* data, uint64_t size, const int32_t* posv, int npos, int control_num, const double* mat);
int qor_apply_named(double* data, uint64_t size, int kind, const int32_t* qubits, const double* params);
int qor_apply_matrix(double* data, uint64_t size, const int32_t* posv, int npos, int control_num, const double* mat);
double qor_expect_pauli(const double* data, uint64_t size, uint64_t x_mask, uint64_t z_mask, int y_count);
void qor_sample_indices(const double* data, uint64_t size, const double* uniforms, int64_t shots, uint64_t* out);
void qor_sample_indices_sorted(const double* data, uint64_t size, const double* uniforms, const int64_t* order,
                               int64_t shots, uint64_t* out);
void qor_sequential_cdf(const double* data, uint64_t size, double* cdf);

#ifdef __cplusplus
}
#endif
#endif
