/*
 * qvnt_oracle.h - CPU restatement of qvnt 0.4.4's state-vector arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU engine is compared with; only the test
 * suite, the smoke check and the CPU-baseline leg of the benchmark load it.  The product library
 * never links or calls it.
 *
 * Every function follows the reference file:line it names, in the same operand order and the
 * same association, without FMA contraction, so that non-fused GPU results are comparable
 * bit for bit.  Gates use the `qvnt_gate` layout of the public header (the data format only).
 *
 * Parity pin: the restatement is checked against the known answers in qvnt's own unit tests
 * (every atomic `matrix_repr`, `quantum_reg`, `tensor`, `wrong_ctrl_mask`, `bits_iter`, `ops`);
 * those values are committed as fixtures with the script that states them.
 */
#ifndef QVNT_ORACLE_H
#define QVNT_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#include "../include/qvnt_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    double re, im;
} oc_t;

/* `AtomicOp::atomic_op(psi, idx)` for every kind (src/operator/atomic/<gate>.rs). */
oc_t oracle_atomic(const qvnt_gate* g, const oc_t* psi, uint64_t idx);
/* `SingleOp::act` = `acts_on()` of the atomic op (u2 returns only a_mask, u2.rs:70-72). */
uint64_t oracle_acts_on(const qvnt_gate* g);
/* `AtomicOp::for_each` (dispatch.rs:32-47) / `for_each_par` (dispatch.rs:50-67) for nthreads > 1. */
void oracle_for_each(const qvnt_gate* g, const oc_t* psi_i, oc_t* psi_o, uint64_t len, int nthreads);
/* `MultiOp::apply{,_sync}` (multi/mod.rs:97-114) through `QReg::apply` (quant.rs:376-395):
 * one out-of-place pass per gate, ping-pong, result left in psi.  scratch: len amplitudes. */
void oracle_apply(const qvnt_gate* gates, size_t count, oc_t* psi, oc_t* scratch, uint64_t len,
                  int nthreads);

/* Register helpers (src/register/quant.rs). len = max(2^n, 8). */
uint64_t oracle_reg_len(uint32_t q_num);
void oracle_reg_init(uint32_t q_num, uint64_t state, oc_t* psi);                 /* :129-150 */
double oracle_get_absolute(const oc_t* psi, uint64_t len);                        /* :458-466 */
void oracle_get_probabilities(const oc_t* psi, uint64_t len, uint32_t q_num, double* out); /* :434-454 */
/* WeightedIndex selection with an injected draw u01 in [0,1) (rand 0.8.5 WeightedIndex::sample). */
uint64_t oracle_weighted_index(const double* w, uint64_t count, double u01);
void oracle_collapse_mask(oc_t* psi, uint64_t len, uint64_t idy, uint64_t mask);  /* :468-486 */
uint64_t oracle_measure_mask(oc_t* psi, uint64_t len, uint32_t q_num, uint64_t mask, double u01,
                             uint64_t* chosen_idx);                               /* :490-501 */
void oracle_reset(oc_t* psi, uint64_t len, uint32_t q_num, uint64_t state);       /* :202-205 */
void oracle_normalize(oc_t* psi, uint64_t len, uint32_t q_num);                   /* :397-414 */
void oracle_reset_by_mask(oc_t* psi, uint64_t len, uint32_t q_num, uint64_t mask);/* :207-229 */
void oracle_get_polar(const oc_t* psi, uint32_t q_num, double* out);              /* :417-431 */
/* Tensor product (quant.rs:330-371); out has oracle_reg_len(na + nb) amplitudes. */
void oracle_tensor(const oc_t* a, uint32_t na, const oc_t* b, uint32_t nb, oc_t* out);
/* `Reg::sample_all(count)` (quant.rs:513-594) with the standard-normal draws injected: z[i], i < 2^n.
 * out gets 2^n counts.  Returns -1 where qvnt panics (n < 3: its probability vector is shorter than
 * the padded buffer it indexes), else 0. */
int oracle_sample_all(const oc_t* psi, uint64_t len, uint32_t q_num, uint64_t count, const double* z,
                      uint64_t* out);
/* `Reg::combine_with_unitary((a, b), c)` (quant.rs:273-308) for two registers of n qubits: out has
 * oracle_reg_len(n + 1) amplitudes; c is a 2x2 complex matrix, interleaved (re, im). */
void oracle_combine_with_unitary(const oc_t* a, const oc_t* b, uint32_t n, const double* c, oc_t* out);
/* `Reg::linear_composition(psi, (c0, c1))` (quant.rs:311-328): self = self * c0 + psi * c1. */
void oracle_linear_composition(oc_t* self, const oc_t* psi, uint64_t len, const double* c);

/* Builders (src/operator/...).  List builders return the number of gates; out may be NULL. */
int oracle_gate_make(uint32_t kind, uint64_t a_mask, uint64_t b_mask, double angle,
                     const double* matrix, qvnt_gate* out);
/* `is_unitary_m1` / `is_unitary_m2` (src/math/matrix.rs:24-73); matrix interleaved (re, im). */
int oracle_is_unitary_m1(const double* m);
int oracle_is_unitary_m2(const double* m);
void oracle_gate_dgr(qvnt_gate* g);
int oracle_gate_c(qvnt_gate* g, uint64_t c_mask);
size_t oracle_op_h(uint64_t mask, qvnt_gate* out);
size_t oracle_op_qft(uint64_t mask, qvnt_gate* out);
size_t oracle_op_qft_swapped(uint64_t mask, qvnt_gate* out);
size_t oracle_op_u3(double the, double phi, double lam, uint64_t mask, qvnt_gate* out);
void oracle_ops_dgr(qvnt_gate* gates, size_t count);
/* `Applicable::matrix(size)` (applicable.rs:17-46); out: (2^size)^2 complex, row-major. */
void oracle_matrix(const qvnt_gate* gates, size_t count, uint32_t size, oc_t* out);

/* OpenMP threads available to the oracle (1 if built without OpenMP). */
int oracle_max_threads(void);

#ifdef __cplusplus
}
#endif

#endif
