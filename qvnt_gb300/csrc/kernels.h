// Host-side launch functions of the engine's kernels.  All run asynchronously on `stream`.
// `fmt` is the register's storage format: FMT_F64 (IEEE f64, plain engine), FMT_DF64 (double-float
// pairs, fused engine), both 16 bytes per amplitude, or FMT_C32 (complex<f32>, 8 bytes, precision
// engine).
#pragma once

#include "common.cuh"

namespace qvnt {

enum Fmt { FMT_F64 = 0, FMT_DF64 = 1, FMT_C32 = 2 };
inline uint64_t fmt_bytes(int fmt) { return fmt == FMT_C32 ? 8 : 16; }

// ---- per-gate passes (gates_plain.cu) ----
bool plain_gate_is_identity(const DevGate& g);
bool plain_gate_needs_gather(const DevGate& g);
int launch_plain_gate(double2* psi, int fmt, uint64_t len, const DevGate& g, cudaStream_t stream,
                      const Geometry& geo);
int launch_gather_gate(const double2* in, double2* out, int fmt, uint64_t len, const DevGate& g, cudaStream_t stream,
                       const Geometry& geo);

// ---- reductions, measurement and register-wide passes (measure.cu) ----
// Number of amplitudes one reduction block covers; partial-sum buffers hold len / kChunk entries.
constexpr uint64_t kChunk = 4096;
inline uint64_t chunk_count(uint64_t len) { return (len + kChunk - 1) / kChunk; }

// Sum of |psi_i|^2 over [0, len) into *d_out (device), deterministic order.  scratch: chunk_count(len)
// doubles.
int launch_norm_sqr_sum(const double2* psi, int fmt, uint64_t len, double* scratch, double* d_out, cudaStream_t stream);
// Full measure_mask on the device: the result index goes to *d_idx (device, 1 uint64).
// scratch: 2 * chunk_count(len) + 8 doubles.  *d_status (device int) gets QVNT_ERR_BAD_ARG when the
// state has zero norm.
int launch_measure(double2* psi, int fmt, uint64_t len, uint64_t q_size, uint64_t mask, double u01, double* scratch,
                   uint64_t* d_idx, int* d_status, int renormalise, cudaStream_t stream);
int launch_inv(const double* d_abs, double* d_inv, int* d_status, cudaStream_t stream);
// p_i = |psi_i|^2 * inv_abs for i in [first, first + count), to d_out.
int launch_probabilities(const double2* psi, int fmt, uint64_t first, uint64_t count, const double* d_inv_abs,
                         double* d_out, cudaStream_t stream);
// (|psi_i|, arg psi_i) for i in [first, first + count), interleaved to d_out.
int launch_polar(const double2* psi, int fmt, uint64_t first, uint64_t count, double* d_out, cudaStream_t stream);
// Amplitudes [first, first + count) as IEEE f64 to d_out / from d_in.
int launch_copy_out(const double2* psi, int fmt, uint64_t first, uint64_t count, double2* d_out, cudaStream_t stream);
int launch_copy_in(double2* psi, int fmt, uint64_t first, uint64_t count, const double2* d_in, cudaStream_t stream);
// psi = |state>.
int launch_reset(double2* psi, int fmt, uint64_t len, uint64_t state, cudaStream_t stream);
// psi_i = 0 where i & mask != 0.
int launch_zero_mask(double2* psi, int fmt, uint64_t len, uint64_t mask, cudaStream_t stream);
// `normalize` (quant.rs:397-414) given d_abs = sum |psi|^2 on the device.
int launch_normalize(double2* psi, int fmt, uint64_t len, const double* d_abs, cudaStream_t stream);
// out_i = a[i & ma] * b[(i >> na) & mb] for i < 2^(na+nb), 0 above (quant.rs:330-371).
int launch_tensor(const double2* a, int fa, uint32_t na, const double2* b, int fb, uint32_t nb, double2* out, int fo,
                  uint64_t out_len, cudaStream_t stream);
// In-place storage conversion: to_df != 0: f64 -> df64, else df64 -> f64.
int launch_convert(double2* psi, uint64_t len, int to_df, cudaStream_t stream);
// Out-of-place conversion between any two formats (dst may not alias src).
int launch_convert_fmt(const double2* src, int fsrc, double2* dst, int fdst, uint64_t len, cudaStream_t stream);
// psi *= sqrt(*d_target / *d_current) (restores a norm after rounding drift; nothing when either is 0).
int launch_rescale(double2* psi, int fmt, uint64_t len, const double* d_target, const double* d_current,
                   cudaStream_t stream);
// sample_all's device part: d_n[i] (q_size doubles) ends as the int64 counts before the host's
// total correction; d_z: injected standard normals (q_size) or null for seeded draws;
// scratch: chunk_count(q_size) doubles; *d_nsum gets the sum of the noise terms.
int launch_sample_all(const double2* psi, int fmt, uint64_t q_size, const double* d_inv, const double* d_z,
                      uint64_t seed, uint64_t count, double* d_n, double* scratch, double* d_nsum,
                      cudaStream_t stream);
// combine_with_unitary: out (out_len) from a, b of n qubits and the 2x2 complex c (interleaved).
int launch_combine(const double2* a, int fa, const double2* b, int fb, uint32_t n, const double* c, double2* out,
                   int fo, uint64_t out_len, cudaStream_t stream);
// linear_composition: self = self * c[0] + psi * c[1] (c: two complex numbers, interleaved).
int launch_linear(double2* self, int fs, const double2* psi, int fp, uint64_t len, const double* c,
                  cudaStream_t stream);
// <a|b> (re, im), <a|a>, <b|b> and max_i |a_i - b_i| into d_out[0..4]; scratch: 5 * chunk_count(len).
int launch_overlap(const double2* a, int fa, const double2* b, int fb, uint64_t len, double* scratch, double* d_out,
                   cudaStream_t stream);

}  // namespace qvnt
