/*
 * qvnt_gb300.h - C ABI of the GB300 state-vector engine for qvnt.
 *
 * The engine replaces the state-owning half of qvnt's `QReg` and the per-amplitude
 * gate loops under it (qvnt 0.4.4):
 *   - `trait Applicable { apply; apply_sync; act_on; dgr; c }`  src/operator/applicable.rs:5-15
 *   - `QReg::{new, with_state, apply, measure_mask, get_probabilities, get_absolute, get_polar}`
 *                                                                src/register/quant.rs:113-505
 *   - `AtomicOp::for_each{,_par}` over the 20 atomic gates      src/operator/atomic/dispatch.rs:28-105
 *
 * A host that keeps qvnt's own circuit building (Rust `op::`, `MultiOp`, `SingleOp`) lowers each
 * `SingleOp{act, ctrl, func}` (src/operator/single/mod.rs:42-47) to one `qvnt_gate` and hands the
 * queue to `qvnt_reg_apply`.  The state vector lives only in GPU memory; there is no CPU path.
 *
 * Conventions
 *   - Every function returns a status code (`QVNT_OK` = 0).  No exception or abort crosses the ABI.
 *     `qvnt_last_error()` returns a thread-local message for the last failing call on this thread.
 *   - Amplitude index i is the basis state |i>, qubit q is bit q of i (LSB = qubit 0).
 *   - Host amplitude buffers are interleaved (re, im) doubles, `Complex<f64>` layout.
 *   - A register holds `max(2^n, 8)` amplitudes, as `QReg` does (src/register/quant.rs:15, :113-150).
 *   - One register maps to one CUDA stream.  A register handle is not thread-safe; different
 *     registers may be used from different threads.
 */
#ifndef QVNT_GB300_H
#define QVNT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------------------------------
 * Status codes.  qvnt panics (`expect`, index out of bounds) or returns `None` where these are
 * returned instead (src/operator/mod.rs:151-155, src/operator/single/mod.rs:4-11, :108-118).
 * ------------------------------------------------------------------------------------------- */
enum qvnt_status {
    QVNT_OK = 0,
    QVNT_ERR_OOM = 1,         /* device allocation failed                                    */
    QVNT_ERR_BAD_MASK = 2,    /* mask outside the register, wrong bit count, ctrl overlaps act */
    QVNT_ERR_BAD_HANDLE = 3,  /* null or destroyed handle                                    */
    QVNT_ERR_CUDA = 4,        /* CUDA runtime error (message in qvnt_last_error)             */
    QVNT_ERR_TIMEOUT = 5,     /* a bounded device wait ran out                               */
    QVNT_ERR_BAD_ARG = 6,     /* other invalid argument (null pointer, bad kind, size)       */
    QVNT_ERR_UNSUPPORTED = 7, /* operation not supported by the engine                       */
    QVNT_ERR_BUSY = 8         /* serving: the admission queue is full, the request was shed   */
};

/* ---------------------------------------------------------------------------------------------
 * Gate kinds, numbered in the order of `enum AtomicOpDispatch` (src/operator/atomic/dispatch.rs:82-105).
 * ------------------------------------------------------------------------------------------- */
enum qvnt_gate_kind {
    QVNT_GATE_ID = 0,          /* atomic/id.rs                                        */
    QVNT_GATE_X = 1,           /* atomic/x.rs    any mask, one pass                   */
    QVNT_GATE_RX = 2,          /* atomic/rx.rs   1-bit mask                           */
    QVNT_GATE_RXX = 3,         /* atomic/rxx.rs  2-bit mask                           */
    QVNT_GATE_Y = 4,           /* atomic/y.rs    any mask                             */
    QVNT_GATE_RY = 5,          /* atomic/ry.rs   1-bit mask                           */
    QVNT_GATE_RYY = 6,         /* atomic/ryy.rs  2-bit mask                           */
    QVNT_GATE_Z = 7,           /* atomic/z.rs    any mask                             */
    QVNT_GATE_S = 8,           /* atomic/s.rs    any mask, dagger flag                */
    QVNT_GATE_T = 9,           /* atomic/t.rs    any mask, dagger flag                */
    QVNT_GATE_RZ = 10,         /* atomic/rz.rs   1-bit mask                           */
    QVNT_GATE_RZZ = 11,        /* atomic/rzz.rs  2-bit mask                           */
    QVNT_GATE_U1 = 12,         /* atomic/u1.rs   1-bit mask, dense 2x2                */
    QVNT_GATE_U2 = 13,         /* atomic/u2.rs   a_mask + b_mask, dense 4x4           */
    QVNT_GATE_H1 = 14,         /* atomic/h1.rs   1-bit mask                           */
    QVNT_GATE_H2 = 15,         /* atomic/h2.rs   a_mask + b_mask (1 bit each)         */
    QVNT_GATE_SWAP = 16,       /* atomic/swap.rs 2-bit mask                           */
    QVNT_GATE_ISWAP = 17,      /* atomic/i_swap.rs 2-bit mask, dagger flag            */
    QVNT_GATE_SQRT_SWAP = 18,  /* atomic/sqrt_swap.rs 2-bit mask, dagger flag         */
    QVNT_GATE_SQRT_ISWAP = 19, /* atomic/sqrt_i_swap.rs 2-bit mask, dagger flag       */
    QVNT_GATE_KIND_COUNT = 20
};

/* One lowered `SingleOp` (src/operator/single/mod.rs:42-47): the atomic function plus its control
 * mask.  Fields a gate kind does not use must be zero.
 *   a_mask  X/Y/Z/S/T/RX/RY/RZ/H1/U1: the `a_mask`;  RXX/RYY/RZZ/SWAP/ISWAP/SQRT_*: the `ab_mask`;
 *           H2/U2: the `a_mask` (one bit).
 *   b_mask  H2/U2 only: the `b_mask` (one bit).
 *   ctrl    `SingleOp::ctrl`: the gate acts where all ctrl bits are 1 (dispatch.rs:35).
 *   dagger  S/T/ISWAP/SQRT_SWAP/SQRT_ISWAP: the `dagger` field of the atomic op.
 *   phase   RX/RY/RZ/RXX/RYY/RZZ: the STORED phase (cos(theta/2), sin(theta/2)) after any `.dgr()`,
 *           which negates both parts (rx.rs:10-14, :42-47).  Carrying the stored phase keeps qvnt's
 *           `.dgr()` semantics, -R(theta), exactly.
 *   matrix  U1: 2x2, U2: 4x4 complex matrix, row-major, interleaved (re, im) (u1.rs:17-25, u2.rs:22-49).
 */
typedef struct qvnt_gate {
    uint32_t kind;
    uint32_t dagger;
    uint64_t a_mask;
    uint64_t b_mask;
    uint64_t ctrl;
    double phase[2];
    double matrix[32];
} qvnt_gate;

typedef struct qvnt_ctx qvnt_ctx;
typedef struct qvnt_reg qvnt_reg;

/* Engines a register can run its gate queue on (a context's default: TENSOR64).
 *   FUSED  groups runs of gates into fused passes staged through shared memory, in double-float
 *          (pairs of FP32, 48-bit significand).
 *   PLAIN  runs one in-place FP64 pass per `SingleOp`, in qvnt's own operand order; its amplitudes
 *          are bit-identical to qvnt's non-fast-math arithmetic.  It is the plain f64 GPU path.
 *   PRECISION keeps complex<f32> amplitudes (8 B) and fuses runs of gates into dense 5-qubit blocks
 *          (32 x 32 complex) contracted on the tensor cores (TF32 split hi + lo, FP32 accumulation);
 *          norms, probabilities and measurement stay FP64.  Registers of at least 12 qubits; gates
 *          whose targets and controls span more than 5 qubits are rejected (QVNT_ERR_UNSUPPORTED).
 *   TENSOR64 keeps IEEE f64 amplitudes (the PLAIN layout) between calls and fuses runs of gates into
 *          dense 5-qubit blocks contracted on the tensor cores: both operands split into exact fp16
 *          digit products (FP32 accumulation of integers below 2^23, no rounding).  Between the passes
 *          of one call the state is 64-bit block floating point (int64 components, one exponent per
 *          register), rounded once per pass to 2^-54 of its largest component; components below about
 *          2^-54 of the largest are not resolved (IEEE f64 would keep them).  Gates spanning more than
 *          5 qubits with their controls, and registers below 12 qubits, run on the PLAIN kernels.
 *          Within 1e-12 of the PLAIN engine. */
enum qvnt_engine { QVNT_ENGINE_FUSED = 0, QVNT_ENGINE_PLAIN = 1, QVNT_ENGINE_PRECISION = 2, QVNT_ENGINE_TENSOR64 = 3 };

/* ---------------------------------------------------------------------------------------------
 * Status / errors
 * ------------------------------------------------------------------------------------------- */
const char* qvnt_status_string(int status);
/* Message of the last failing call on the calling thread ("" if none). */
const char* qvnt_last_error(void);
/* ABI version: (major << 16) | minor. */
uint32_t qvnt_abi_version(void);

/* ---------------------------------------------------------------------------------------------
 * Context: one CUDA device.  Replaces the global Rayon pool (src/threads.rs:32-52).
 * ------------------------------------------------------------------------------------------- */
int qvnt_ctx_create(int device, qvnt_ctx** out);
int qvnt_ctx_destroy(qvnt_ctx* ctx);
/* Free device memory and the total in bytes, as the CUDA runtime reports them for this device. */
int qvnt_ctx_mem_info(qvnt_ctx* ctx, uint64_t* free_bytes, uint64_t* total_bytes);
/* Engine (enum qvnt_engine) of the registers qvnt_reg_create makes on this context and of the
 * scratch register of qvnt_apply_host (which runs PRECISION requests on FUSED); default TENSOR64.
 * No counterpart in the reference (its one CPU path has no choice to make). */
int qvnt_ctx_set_engine(qvnt_ctx* ctx, int engine);

/* ---------------------------------------------------------------------------------------------
 * Registers (QReg, src/register/quant.rs:102-150)
 * ------------------------------------------------------------------------------------------- */
/* `QReg::with_state(q_num, state)`; `QReg::new(q_num)` is state = 0.  The state index is masked
 * by 2^q_num - 1 as in quant.rs:131-142.  q_num <= 40. */
int qvnt_reg_create(qvnt_ctx* ctx, uint32_t q_num, uint64_t state, qvnt_reg** out);
/* As qvnt_reg_create, on a chosen engine (enum qvnt_engine): a PRECISION register is allocated at
 * 8 B per amplitude from the start. */
int qvnt_reg_create_ex(qvnt_ctx* ctx, uint32_t q_num, uint64_t state, int engine, qvnt_reg** out);
int qvnt_reg_destroy(qvnt_reg* reg);
/* `QReg::clone` (derive(Clone), quant.rs:102). */
int qvnt_reg_clone(const qvnt_reg* reg, qvnt_reg** out);
/* `QReg::num` (quant.rs:152-154). */
int qvnt_reg_num(const qvnt_reg* reg, uint32_t* q_num);
/* Number of stored amplitudes, max(2^q_num, 8) (quant.rs:15, :116). */
int qvnt_reg_len(const qvnt_reg* reg, uint64_t* len);
/* Select the engine (enum qvnt_engine) that later qvnt_reg_apply calls use. */
int qvnt_reg_set_engine(qvnt_reg* reg, int engine);
/* Fused engine: tile width in qubits (0 = automatic).  Values outside [6, 13] are rejected. */
int qvnt_reg_set_fusion_width(qvnt_reg* reg, uint32_t k);

/* `QReg::apply(&MultiOp)` (quant.rs:376-395, multi/mod.rs:97-114): the gates run in order, each one
 * over the whole register.  All gates are validated before any runs; an invalid gate returns
 * QVNT_ERR_BAD_MASK or QVNT_ERR_BAD_ARG and leaves the state unchanged.  Asynchronous on the
 * register's stream: errors raised by the device surface on the next synchronising call. */
int qvnt_reg_apply(qvnt_reg* reg, const qvnt_gate* gates, size_t count);

/* `QReg::measure_mask(mask)` (quant.rs:490-501) with the uniform draw injected by the caller:
 * u01 in [0, 1) replaces `thread_rng()`.  The chosen index is the first i whose inclusive
 * cumulative probability exceeds u01 * (sum of probabilities), qvnt's `WeightedIndex` rule.
 * Collapses amplitudes with (i ^ idx) & mask != 0 to zero WITHOUT renormalising, as qvnt does.
 * *out_value = idx & mask (`CReg::get`).  mask & (2^n - 1) == 0 returns 0 and leaves the state. */
int qvnt_reg_measure_mask(qvnt_reg* reg, uint64_t mask, double u01, uint64_t* out_value);
/* Same as qvnt_reg_measure_mask, then rescales the state to unit norm when renormalise != 0. */
int qvnt_reg_measure_mask_ex(qvnt_reg* reg, uint64_t mask, double u01, int renormalise,
                             uint64_t* out_value);

/* `QReg::get_probabilities` (quant.rs:434-454): p_i = |psi_i|^2 * (1 / sum over the whole buffer),
 * for i < 2^n.  host_out holds 2^n doubles. */
int qvnt_reg_get_probabilities(qvnt_reg* reg, double* host_out);
/* `QReg::get_absolute` (quant.rs:458-466): sum of |psi_i|^2 over the whole buffer. */
int qvnt_reg_get_absolute(qvnt_reg* reg, double* out);
/* `QReg::get_polar` (quant.rs:417-431): (|psi_i|, arg psi_i) for i < 2^n, interleaved, 2*2^n doubles. */
int qvnt_reg_get_polar(qvnt_reg* reg, double* host_out);
/* Copies all max(2^n, 8) amplitudes to the host, interleaved (re, im). */
int qvnt_reg_get_amplitudes(qvnt_reg* reg, double* host_out);
/* Copies amplitudes [first, first + count) to the host, interleaved (re, im): a slice of qvnt's
 * `psi` without reading the whole state. */
int qvnt_reg_get_amplitudes_range(qvnt_reg* reg, uint64_t first, uint64_t count, double* host_out);
/* Replaces all max(2^n, 8) amplitudes from the host, interleaved (re, im). */
int qvnt_reg_set_amplitudes(qvnt_reg* reg, const double* host_in);
/* `QReg::reset(state)` (quant.rs:202-205): |state & q_mask>. */
int qvnt_reg_reset(qvnt_reg* reg, uint64_t state);
/* `QReg::reset_by_mask(mask)` (quant.rs:207-229): zero amplitudes with i & mask != 0, then
 * `normalize` (quant.rs:397-414); mask covering all qubits resets to |0>. */
int qvnt_reg_reset_by_mask(qvnt_reg* reg, uint64_t mask);
/* `normalize` (quant.rs:397-414): norm <= 1e-15 resets to |0>; 1 - norm <= 1e-9 leaves the state. */
int qvnt_reg_normalize(qvnt_reg* reg);
/* Tensor product `QReg * QReg` (quant.rs:330-371): out = a (low qubits) x b (high qubits). */
int qvnt_reg_tensor(const qvnt_reg* a, const qvnt_reg* b, qvnt_reg** out);
/* Waits for all work queued on the register's stream. */
int qvnt_reg_sync(qvnt_reg* reg);
/* The register's cudaStream_t, for callers that order their own work (or timing events) after it. */
int qvnt_reg_get_stream(const qvnt_reg* reg, void** stream);

/* ---------------------------------------------------------------------------------------------
 * Out-of-place plugin call: `Applicable::apply(&self, psi_i: &[C], psi_o: &mut Vec<C>)`
 * (src/operator/applicable.rs:5-6).  psi_i and psi_o are host buffers of `len` interleaved
 * complex doubles (len a power of two, >= 8); the call copies psi_i to the device, runs the gates
 * on the context's scratch register and copies the result to psi_o before returning.
 * ------------------------------------------------------------------------------------------- */
int qvnt_apply_host(qvnt_ctx* ctx, const qvnt_gate* gates, size_t count, const double* psi_i,
                    double* psi_o, uint64_t len);

/* ---------------------------------------------------------------------------------------------
 * Gate builders for hosts without qvnt's Rust `op::` (C, C++, Python).  A Rust host keeps its own
 * `op::` and lowers `SingleOp`s itself.  List builders write at most `cap` gates to `out` and the
 * full count to *count; call with cap = 0 to size the list.
 * ------------------------------------------------------------------------------------------- */
/* Checked single-gate constructor, the atomic `::new` + `is_valid` (single/mod.rs:4-11).
 * angle is used by RX/RY/RZ/RXX/RYY/RZZ (stored as (cos(angle/2), sin(angle/2)));
 * matrix (8 or 32 doubles) by U1/U2.  Invalid masks return QVNT_ERR_BAD_MASK. */
int qvnt_gate_make(uint32_t kind, uint64_t a_mask, uint64_t b_mask, double angle,
                   const double* matrix, qvnt_gate* out);
/* `SingleOp::dgr` (single/mod.rs:97-103). */
int qvnt_gate_dgr(qvnt_gate* gate);
/* `SingleOp::c` (single/mod.rs:106-116): QVNT_ERR_BAD_MASK if c_mask overlaps act | ctrl. */
int qvnt_gate_c(qvnt_gate* gate, uint64_t c_mask);
/* `SingleOp::act_on` = act | ctrl (single/mod.rs:93-95). */
uint64_t qvnt_gate_act_on(const qvnt_gate* gate);
/* `SingleOp::name` (single/mod.rs:72-78), e.g. "C8_H3", "RX1(1.23456)".  Writes at most cap bytes
 * including the terminator; *needed gets the full length without it. */
int qvnt_gate_name(const qvnt_gate* gate, char* buf, size_t cap, size_t* needed);
/* `op::h(mask)` (src/operator/multi/h.rs:14-45): H2 over pairs of set bits, then H1 if odd. */
int qvnt_op_h(uint64_t mask, qvnt_gate* out, size_t cap, size_t* count);
/* `op::qft(mask)` (src/operator/multi/qft.rs:4-33): H then controlled RZ(pi/2^j), no swaps. */
int qvnt_op_qft(uint64_t mask, qvnt_gate* out, size_t cap, size_t* count);
/* `op::qft_swapped(mask)` (src/operator/multi/qft.rs:35-52). */
int qvnt_op_qft_swapped(uint64_t mask, qvnt_gate* out, size_t cap, size_t* count);
/* `op::u2(phi, lam, mask)` = rz(lam) ry(pi/2) rz(phi) (src/operator/mod.rs:480-482), 3 gates. */
int qvnt_op_u2(double phi, double lam, uint64_t mask, qvnt_gate* out, size_t cap, size_t* count);
/* `op::u3(the, phi, lam, mask)` = rz(lam) ry(the) rz(phi) (src/operator/mod.rs:499-501), 3 gates. */
int qvnt_op_u3(double the, double phi, double lam, uint64_t mask, qvnt_gate* out, size_t cap,
               size_t* count);
/* `MultiOp::dgr` (multi/mod.rs:120-123): reverses the list and daggers each gate, in place. */
int qvnt_ops_dgr(qvnt_gate* gates, size_t count);
/* `MultiOp::c` (multi/mod.rs:125-132): controls every gate; fails if c_mask overlaps act_on. */
int qvnt_ops_c(qvnt_gate* gates, size_t count, uint64_t c_mask);

/* ---------------------------------------------------------------------------------------------
 * Wire formats for gate lists (host only, no device work).
 *
 * Text: `MultiOp`'s `{:?}` (src/operator/multi/mod.rs:90-94), a list of `SingleOp::name`s
 * (single/mod.rs:72-78) such as "[C4_X123, RX1(1.23456), U1[[Complex { re: 1.0, im: 0.0 }, ...]]]".
 *   qvnt_ops_name   writes that text for a gate list (at most cap bytes with the terminator;
 *                   *needed = the full length without it).
 *   qvnt_ops_parse  reads it back (or one bare name): `len` bytes, no terminator needed; the
 *                   gates are built as the qvnt constructors build them (qvnt_gate_make,
 *                   qvnt_gate_c), so masks and unitarity are checked.  At most cap gates are
 *                   written, *count = all of them.  QVNT_ERR_BAD_ARG names the byte offset of a
 *                   syntax error.  qvnt's names do not hold everything a gate does: S, T, iSWAP,
 *                   sqrt(SWAP) and sqrt(iSWAP) print no dagger (parsed: not daggered); a rotation
 *                   prints 2 arg(phase) (parsed: the gate qvnt_gate_make builds for that angle);
 *                   U2 prints a | b (parsed: a the lower bit, b the higher); non-finite numbers are
 *                   rejected.  The binary form below keeps every bit.
 *
 * Binary: a versioned, CRC-32-checked little-endian stream holding every field of each gate bit
 * for bit, alone (gates) or with the rest of a serving request (q_num, state, submit flags and the
 * calls of qvnt_server_submit).  Encoders write the stream only when it fits (cap >= *len) and
 * always set *len; decoders reject a bad magic, version, type, CRC, truncation, unknown fields or
 * trailing bytes with QVNT_ERR_BAD_ARG, write at most cap records and set the full counts (call
 * with cap = 0 to size the buffers).  A request's APPLY calls must take exactly its gate list.
 * ------------------------------------------------------------------------------------------- */
int qvnt_ops_name(const qvnt_gate* gates, size_t count, char* buf, size_t cap, size_t* needed);
int qvnt_ops_parse(const char* text, size_t len, qvnt_gate* out, size_t cap, size_t* count);
int qvnt_wire_encode_gates(const qvnt_gate* gates, size_t count, uint8_t* buf, size_t cap, size_t* len);
int qvnt_wire_decode_gates(const uint8_t* buf, size_t len, qvnt_gate* out, size_t cap, size_t* count);

/* Plans a gate list for a q_num-qubit register on the fused engine without running it (host only,
 * no device work): the number of passes (HBM round trips), register stages and engine gates it
 * lowers to.  fusion_k as for qvnt_reg_set_fusion_width (0 = automatic). */
int qvnt_plan_info(const qvnt_gate* gates, size_t count, uint32_t q_num, uint32_t fusion_k, uint64_t* passes,
                   uint64_t* stages, uint64_t* engine_gates);

/* ---------------------------------------------------------------------------------------------
 * Allocation-free norm.  No counterpart in the reference: an extra entry point for callers that
 * cannot call cudaMalloc -- hosts whose device memory is owned by their own allocator or pool (a
 * framework's caching allocator, a serving process with a fixed memory budget), and code paths
 * where cudaMalloc/cudaFree would synchronise the device in the middle of their stream work.
 *
 * Sum of |psi_i|^2 over a state vector the caller keeps in device memory: d_psi holds len
 * interleaved (re, im) IEEE f64 amplitudes and must be 16-byte aligned (it is read as double2); the
 * sum is written to the device double *d_out (8-byte aligned).  Misaligned pointers are refused with
 * QVNT_ERR_BAD_ARG before anything is queued.  The
 * kernels are queued on `stream` (a cudaStream_t; NULL = the legacy default stream) and the call
 * returns without waiting.  It allocates nothing: its partial sums live in a file-scope device
 * array of QVNT_NOALLOC_MAX_AMPLITUDES / 4096 doubles (512 KiB) that every GPU loading the library
 * holds until the process exits; len above QVNT_NOALLOC_MAX_AMPLITUDES (2^28, a 28-qubit state) is
 * rejected with QVNT_ERR_BAD_ARG.  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress, with that device current); make that first call before any stream
 * capture.  All calls on a device share the array: calls that overlap on the GPU (different
 * streams, no ordering between them) race on it.  Same reduction order as qvnt_reg_get_absolute.
 * ------------------------------------------------------------------------------------------- */
#define QVNT_NOALLOC_MAX_AMPLITUDES (1ull << 28)
int qvnt_norm_sqr_noalloc(const double* d_psi, uint64_t len, double* d_out, void* stream);

/* ---------------------------------------------------------------------------------------------
 * Counters for measurement: kernels launched and fused passes run by this register so far.
 * ------------------------------------------------------------------------------------------- */
int qvnt_reg_stats(const qvnt_reg* reg, uint64_t* kernel_launches, uint64_t* passes);
/* `Reg::sample_all(count)` (src/register/quant.rs:513-594): a histogram of `count` measurements
 * without collapse, p_i count plus Gaussian noise, corrected to sum to `count`.  out_counts gets 2^n
 * entries.  `normals` (2^n standard normal draws, host memory) replaces qvnt's thread_rng draws when
 * given; otherwise the draws come from `seed` on the device.  Registers below 3 qubits are rejected
 * (qvnt panics there: its probability vector is shorter than the padded buffer it walks). */
int qvnt_reg_sample_all(qvnt_reg* reg, uint64_t count, uint64_t seed, const double* normals, uint64_t* out_counts);
/* `Reg::combine_with_unitary((a, b), c)` (quant.rs:273-308): a new register of n + 1 qubits whose lower
 * half is c00 a + c01 b and upper half c10 a + c11 b; c is a unitary 2x2 complex matrix, interleaved. */
int qvnt_reg_combine_with_unitary(const qvnt_reg* a, const qvnt_reg* b, const double* c, qvnt_reg** out);
/* `Reg::linear_composition(psi, (c0, c1))` (quant.rs:311-328): self = self * c0 + psi * c1; c holds
 * c0 and c1 interleaved (re, im). */
int qvnt_reg_linear_composition(qvnt_reg* self, const qvnt_reg* psi, const double* c);
/* State comparison in FP64 across engines (no counterpart in the reference): fidelity
 * |<a|b>|^2 / (<a|a> <b|b>) and max_i |a_i - b_i|.  Registers of the same size and context. */
int qvnt_reg_overlap(const qvnt_reg* a, const qvnt_reg* b, double* fidelity, double* max_abs_diff);
/* Host-side plan of the precision engine for a gate list on q_num (>= 12) qubits: passes and dense
 * 5-qubit blocks. */
int qvnt_precision_plan_info(const qvnt_gate* gates, size_t count, uint32_t q_num, uint64_t* passes,
                             uint64_t* blocks);
/* Host-side plan of the TENSOR64 engine for a gate list on q_num qubits: tensor-core passes (one
 * dense 5-qubit block each) and gates left to single PLAIN passes (no counterpart in the reference). */
int qvnt_tensor64_plan_info(const qvnt_gate* gates, size_t count, uint32_t q_num, uint64_t* passes,
                            uint64_t* plain_gates);
/* The dense 5-qubit blocks the TENSOR64 engine would run for a gate list on q_num (>= 5) qubits, in
 * order (the planner of the tensor and precision engines; no counterpart in the reference).  Every gate
 * must span at most 5 qubits with its controls (else QVNT_ERR_UNSUPPORTED).  *nblocks = the number of
 * blocks; when cap >= *nblocks, sups[i] = block i's 5 qubits (a mask) and mats[2048 i ...] its 32 x 32
 * unitary, row-major, interleaved (re, im), local bit j = the j-th lowest qubit of sups[i]. */
int qvnt_dense_plan_blocks(const qvnt_gate* gates, size_t count, uint32_t q_num, uint64_t* sups, double* mats,
                           size_t cap, size_t* nblocks);
/* The cost, in SM cycles, of the TENSOR64 pass's tensor-core instructions measured in isolation on
 * every SM of the context's device: one tcgen05.mma.kind::f16 (M = 128, K = 16) of N = 64 and of
 * N = 256, and the 44 MMAs of one pass tile (the pass's mix of N = 64 .. 256).  A measurement, not
 * part of the path. */
int qvnt_tensor64_mma_costs(qvnt_ctx* ctx, double* n64_cycles, double* n256_cycles, double* tile_cycles);
/* Time the fused engine spends in its dominant kernel: CUDA events recorded around every launch of
 * the fused-pass kernel on the register's stream since the last reset (enable != 0 turns
 * recording on and clears the totals).  *ms = summed event time, *launches = number of launches. */
int qvnt_reg_kernel_timing(qvnt_reg* reg, int enable, double* ms, uint64_t* launches);

/* ---------------------------------------------------------------------------------------------
 * Batching form: many independent registers in one persistent launch.  Each register behaves as
 * `QReg::with_state(q_nums[i], states[i])` (src/register/quant.rs:113-150) followed by `apply` of its
 * own gate list (quant.rs:376-395) and, when measure_masks[i] != 0, `measure_mask(measure_masks[i])`
 * (quant.rs:490-501, collapse without renormalisation).  The replacement for a caller looping over
 * registers on the host; qvnt itself has no batch object.
 *
 *   qvnt_batch_create   copies the circuits (gate_offsets[i]..gate_offsets[i+1] of `gates` belong to
 *                       register i; count + 1 offsets), validates every gate against its register,
 *                       allocates the states (double-float, 16 B per amplitude), plans the schedule
 *                       and captures one run as a CUDA graph.  4 <= q_nums[i] <= 26.  Gates that the
 *                       fused tile engine does not take (a U2 whose control overlaps its b bit) are
 *                       rejected with QVNT_ERR_UNSUPPORTED.
 *   qvnt_batch_run      replays the graph: states reset to their basis states, every circuit applied,
 *                       every measurement taken with its injected draw u01[i] in [0, 1) (required when
 *                       any mask is non-zero); measured[i] = the CReg value (0 where the mask is 0).
 *   qvnt_batch_set_fusion / qvnt_batch_autotune
 *                       re-plan with a tile width (fusion_k, 6..12) and pass budget (estimated FP32
 *                       instructions per amplitude a pass may hold; 0 = the engine default), or pick
 *                       both, and the kernel's register budget (2 CTAs per SM or 1 without spills), by
 *                       timing the schedule of every stride-th register under each candidate.
 *   qvnt_batch_get_amplitudes  register `index` after the last run, interleaved (re, im) f64.
 *   qvnt_batch_info     schedule items and passes, state bytes, fusion width, pass budget, and the
 *                       device time of the last run (events around the graph launch).
 * ------------------------------------------------------------------------------------------- */
/* Seeded synthetic layers for the batch and serving workloads (no counterpart in the reference):
 * per layer one gate from {h, s, t, u3} on every qubit, 15 gates from {rxx, ryy, rzz, swap, i_swap,
 * sqrt_i_swap} on random distinct pairs and 3 Toffolis, drawn from the SplitMix64 state
 * *rng_state, which is advanced in place (also when cap is too small: gates are then only counted).
 * Same draws, same gates as the Python generator qvnt_gb300.circuits.random_layers. */
int qvnt_workload_random_layers(uint32_t n, uint32_t depth, uint64_t* rng_state, qvnt_gate* out, size_t cap,
                                size_t* count);

typedef struct qvnt_batch qvnt_batch;
int qvnt_batch_create(qvnt_ctx* ctx, uint32_t count, const uint32_t* q_nums, const uint64_t* states,
                      const qvnt_gate* gates, const uint64_t* gate_offsets, const uint64_t* measure_masks,
                      qvnt_batch** out);
int qvnt_batch_destroy(qvnt_batch* batch);
int qvnt_batch_run(qvnt_batch* batch, const double* u01, uint64_t* measured);
int qvnt_batch_set_fusion(qvnt_batch* batch, uint32_t fusion_k, uint32_t pass_budget);
int qvnt_batch_autotune(qvnt_batch* batch, uint32_t stride, uint32_t* fusion_k, uint32_t* pass_budget,
                        double* best_ms);
int qvnt_batch_get_amplitudes(qvnt_batch* batch, uint32_t index, double* out);
int qvnt_batch_info(const qvnt_batch* batch, uint64_t* items, uint64_t* passes, uint64_t* state_bytes,
                    uint32_t* fusion_k, uint32_t* pass_budget, double* last_ms);

/* ---------------------------------------------------------------------------------------------
 * Serving form: a request loop with continuous admission.  A request is one register's life:
 * `QReg::with_state(q_num, state)` (src/register/quant.rs:113-150), then its calls in order on the
 * resident state -- QVNT_CALL_APPLY applies the next `gate_count` gates of the request's gate list
 * (`QReg::apply`, quant.rs:376-395), QVNT_CALL_MEASURE is `measure_mask(mask)` with the injected draw
 * u01 (quant.rs:490-501).  No counterpart in the reference, whose QReg is driven by one caller.
 *
 *   qvnt_server_create   `slots` worker threads; requests are admitted while the states of the
 *                        running ones fit `hbm_budget_bytes` (16 B per amplitude, plus the same again
 *                        for a request that keeps its amplitudes).  Among the queued requests that
 *                        fit, the one with the least work (amplitudes x gates) discounted by
 *                        exp(-waiting seconds) goes next; requests of 24 qubits or more hold at most
 *                        a quarter of the slots (at most 8).  Requests beyond `max_queue` queued ones are shed
 *                        (QVNT_ERR_BUSY; 0 = 4096).
 *   qvnt_server_submit   copies the request (gates validated against the register); `arrival_s` is
 *                        its arrival on the server clock (qvnt_server_clock; < 0 = now), the start of
 *                        its latency.  flags: QVNT_SUBMIT_KEEP_AMPLITUDES keeps the final state for
 *                        qvnt_server_wait; QVNT_SUBMIT_DETACHED releases the request when it completes
 *                        (no wait; its latency still enters the statistics).
 *   qvnt_server_wait     blocks (timeout_s < 0: without limit) until the request completes; results
 *                        gets one value per call (the measured value; 0 for APPLY), amplitudes the
 *                        final state (interleaved f64, max(2^q_num, 8) amplitudes) when kept.
 *   qvnt_server_latencies / qvnt_server_queued_ages
 *                        completion latencies (seconds, in completion order) and the waiting times
 *                        of the requests still queued.
 *   qvnt_server_destroy  finishes the running requests, fails the queued ones; no wait may be in
 *                        progress on another thread.
 * Each slot drives its own CUDA stream: give the process at least as many hardware work queues as
 * slots (CUDA_DEVICE_MAX_CONNECTIONS, at most 32; qvnt_ctx_create sets 32 unless the variable is
 * set), or the kernels of small requests wait in FIFO order behind those of large ones.
 * ------------------------------------------------------------------------------------------- */
#define QVNT_CALL_APPLY 0u
#define QVNT_CALL_MEASURE 1u
#define QVNT_SUBMIT_KEEP_AMPLITUDES 1
#define QVNT_SUBMIT_DETACHED 2

typedef struct qvnt_call {
    uint32_t op;          /* QVNT_CALL_APPLY or QVNT_CALL_MEASURE */
    uint32_t reserved;
    uint64_t gate_count;  /* APPLY: gates taken from the request's list */
    uint64_t mask;        /* MEASURE: mask */
    double u01;           /* MEASURE: uniform draw in [0, 1) */
} qvnt_call;

typedef struct qvnt_server_counters {
    uint64_t submitted, shed, completed, failed, queued, running, peak_running;
    uint64_t bytes_active, bytes_pooled;
    double now_s;
} qvnt_server_counters;

typedef struct qvnt_server qvnt_server;
int qvnt_server_create(qvnt_ctx* ctx, uint64_t hbm_budget_bytes, uint32_t slots, uint32_t max_queue,
                       qvnt_server** out);
int qvnt_server_destroy(qvnt_server* server);
int qvnt_server_clock(qvnt_server* server, double* now_s);
int qvnt_server_submit(qvnt_server* server, uint32_t q_num, uint64_t state, const qvnt_gate* gates,
                       const qvnt_call* calls, uint32_t ncalls, double arrival_s, int flags, uint64_t* id);
int qvnt_server_wait(qvnt_server* server, uint64_t id, double timeout_s, uint64_t* results, double* amplitudes,
                     double* latency_s);
int qvnt_server_stats(qvnt_server* server, qvnt_server_counters* out);
int qvnt_server_latencies(qvnt_server* server, double* out, size_t cap, size_t* count);
int qvnt_server_queued_ages(qvnt_server* server, double* out, size_t cap, size_t* count);

/* ---------------------------------------------------------------------------------------------
 * QASM runner: `Sym::finish` (src/qasm/sym.rs:40-74) on a register.  A program is qvnt's
 * interpreted `int::Op` (src/qasm/int/ext_op.rs:6-16): blocks of gates, each ending in a separator,
 * then `trailing_gates` more gates.  Block b applies the next blocks[b].gate_count gates of `gates`
 * and then, by blocks[b].sep:
 *   QVNT_SEP_NOP      nothing more
 *   QVNT_SEP_MEASURE  measure_mask(a) with the next draw of u01; the k-th set bit of a sets (or, with
 *                     QVNT_MEASURE_XOR, xors) the k-th set bit of b in *creg from the measured bit
 *   QVNT_SEP_IF       the block's gates run only if the bits of *creg under a (within c_num bits),
 *                     packed low to high, equal b (`CReg::get_by_mask`, register/class.rs:115-125)
 *   QVNT_SEP_RESET    reset_by_mask(a)
 * *creg is the classical register (`CReg`, c_num <= 64 bits) on entry and on return; *draws_used
 * the draws taken.  Blocks, gates (against the register) and the draws of every MEASURE block
 * (in [0, 1)) are checked before anything runs; an invalid program changes nothing.
 * No counterpart of the QASM parser (qvnt-qasm) is built: the caller lowers the program.
 * ------------------------------------------------------------------------------------------- */
#define QVNT_SEP_NOP 0u
#define QVNT_SEP_MEASURE 1u
#define QVNT_SEP_IF 2u
#define QVNT_SEP_RESET 3u
#define QVNT_MEASURE_SET 0
#define QVNT_MEASURE_XOR 1

typedef struct qvnt_block {
    uint32_t sep;         /* QVNT_SEP_* */
    uint32_t reserved;
    uint64_t gate_count;  /* gates taken from the program's list */
    uint64_t a;           /* MEASURE: qubit mask; IF: classical mask; RESET: qubit mask */
    uint64_t b;           /* MEASURE: classical mask; IF: value */
} qvnt_block;

int qvnt_program_run(qvnt_reg* reg, uint32_t c_num, int measure_op, const qvnt_gate* gates,
                     const qvnt_block* blocks, uint32_t nblocks, uint64_t trailing_gates, const double* u01,
                     uint32_t nu01, uint64_t* creg, uint32_t* draws_used);

/* A program as text (host only): qvnt's `Debug` of `int::Op` (src/qasm/int/ext_op.rs:77-112), what
 * `Int::get_ops_tree` returns (src/qasm/int/mod.rs:398-400), e.g.
 * "[H3, H4] -> Measure(11 => 11) -> if c[1] == 1 { [X4] } -> [Z4]" (masks in binary).
 *   qvnt_program_format  writes it (at most cap bytes with the terminator; *needed = full length).
 *   qvnt_program_parse   reads it back; gate names as qvnt_ops_parse reads them.  Two gate lists in
 *                        a row make a NOP block; a list before Measure/Reset is that block's gates.
 *                        At most gcap gates and bcap blocks are written, the counts are always set.
 * The text does not show an empty NOP block or where a NOP block ends and the next block's gates
 * begin, so a parsed program may group its gates differently; it runs the same gates in the same
 * order with the same separators, and formats to the same text. */
/* OpenQASM 2.0 source to a program for qvnt_program_run (host only): `Int::new(Ast::from_source(..))`
 * (src/qasm/int/mod.rs:56-60).  Qubits and bits are allocated in declaration order (*q_num, *c_num:
 * the register sizes `Sym::new` uses, at most 64 each); gate names map as qvnt's table does
 * (src/qasm/int/gates.rs:86-126: a leading c/C controls by the first register, registers OR into one
 * mask, sdg/tdg build S/T); `gate` definitions expand with their parameters; arguments are evaluated
 * with pi, sqrt, exp, ln, abs, floor, ceil, round, atan2, max, min (src/qasm/int/parse.rs:5-25);
 * `include` is skipped.  At most gcap gates and bcap blocks are written, the counts always set.
 * Errors (syntax, unknown names, sizes, masks) return QVNT_ERR_BAD_ARG with the reason. */
int qvnt_qasm_compile(const char* source, size_t len, uint32_t* q_num, uint32_t* c_num, qvnt_gate* gates,
                      size_t gcap, size_t* ngates, qvnt_block* blocks, uint32_t bcap, uint32_t* nblocks,
                      uint64_t* trailing_gates);

int qvnt_program_format(const qvnt_gate* gates, const qvnt_block* blocks, uint32_t nblocks, uint64_t trailing_gates,
                        char* buf, size_t cap, size_t* needed);
int qvnt_program_parse(const char* text, size_t len, qvnt_gate* gates, size_t gcap, size_t* ngates,
                       qvnt_block* blocks, uint32_t bcap, uint32_t* nblocks, uint64_t* trailing_gates);

/* A serving request as one binary wire stream (format above qvnt_ops_name): the arguments of
 * qvnt_server_submit except the server and the arrival time.  Host only. */
int qvnt_wire_encode_request(uint32_t q_num, uint64_t state, int flags, const qvnt_gate* gates, size_t ngates,
                             const qvnt_call* calls, uint32_t ncalls, uint8_t* buf, size_t cap, size_t* len);
int qvnt_wire_decode_request(const uint8_t* buf, size_t len, uint32_t* q_num, uint64_t* state, int* flags,
                             qvnt_gate* gates, size_t gcap, size_t* ngates, qvnt_call* calls, uint32_t ccap,
                             uint32_t* ncalls);

#ifdef __cplusplus
}
#endif

#endif /* QVNT_GB300_H */
