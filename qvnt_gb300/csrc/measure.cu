// Register-wide passes: norm, probabilities, measure_mask, collapse, normalize, reset, tensor and
// storage-format conversion.
//
// Every kernel reads amplitudes through an accessor (AccF64: IEEE f64 storage of the plain engine;
// AccDF64: double-float storage of the fused engine) and computes in FP64.  Built with --fmad=false
// so that |psi|^2 = re*re + im*im and p_i = |psi_i|^2 * (1/sum) round as qvnt's `norm_sqr` and
// `get_probabilities` do (src/register/quant.rs:434-454).  Sums are taken in a fixed tree order
// (chunk partials, then one block): results are reproducible run to run.
#include <math.h>

#include <mutex>

#include "atomic.cuh"
#include "df64.cuh"
#include "kernels.h"

namespace qvnt {

namespace {

constexpr int kRedThreads = 256;    // chunk reduction block
constexpr int kScanThreads = 1024;  // single-block search

__device__ __forceinline__ double nsq(double2 z) { return z.x * z.x + z.y * z.y; }

template <int THREADS>
__device__ __forceinline__ double block_sum(double v, double* sm) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sm[w] = v;
    __syncthreads();
    double t = 0.0;
    if (w == 0) {
        t = (l < THREADS / 32) ? sm[l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    return t;  // valid in thread 0
}

// Inclusive scan over the block in thread order; *total gets the block total.
template <int THREADS>
__device__ __forceinline__ double block_inclusive_scan(double v, double* sm, double* total) {
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        double u = __shfl_up_sync(0xffffffffu, v, o);
        if (l >= o) v += u;
    }
    __syncthreads();
    if (l == 31) sm[w] = v;
    __syncthreads();
    if (w == 0) {
        double s = (l < THREADS / 32) ? sm[l] : 0.0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            double u = __shfl_up_sync(0xffffffffu, s, o);
            if (l >= o) s += u;
        }
        if (l < THREADS / 32) sm[l] = s;
    }
    __syncthreads();
    if (w > 0) v += sm[w - 1];
    *total = sm[THREADS / 32 - 1];
    return v;
}

// Partial sums per chunk of kChunk amplitudes: sum_i |psi_i|^2 (* scale) over i < limit.
template <class Acc>
__global__ void __launch_bounds__(kRedThreads) chunk_sum_kernel(const double2* __restrict__ psi, uint64_t limit,
                                                                 const double* __restrict__ d_scale,
                                                                 double* __restrict__ partial) {
    __shared__ double sm[32];
    const uint64_t base = (uint64_t)blockIdx.x * kChunk;
    const double scale = d_scale ? *d_scale : 1.0;
    double s = 0.0;
    for (uint32_t k = threadIdx.x; k < kChunk; k += kRedThreads) {
        const uint64_t i = base + k;
        if (i < limit) s += d_scale ? nsq(Acc::load(psi, i)) * scale : nsq(Acc::load(psi, i));
    }
    double t = block_sum<kRedThreads>(s, sm);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

__global__ void __launch_bounds__(kScanThreads) final_sum_kernel(const double* __restrict__ partial, uint64_t n,
                                                                  double* __restrict__ out) {
    __shared__ double sm[32];
    double s = 0.0;
    for (uint64_t k = threadIdx.x; k < n; k += kScanThreads) s += partial[k];
    double t = block_sum<kScanThreads>(s, sm);
    if (threadIdx.x == 0) *out = t;
}

// inv = 1/abs; flags a zero or non-finite norm (qvnt's WeightedIndex::new(..).unwrap() panics).
__global__ void inv_kernel(const double* d_abs, double* d_inv, int* d_status) {
    const double a = *d_abs;
    *d_inv = 1. / a;
    if (!(a > 0.0) || !isfinite(1. / a)) *d_status = QVNT_ERR_BAD_ARG;
}

// WeightedIndex selection (rand 0.8.5): first i with inclusive cumulative p > u01 * total,
// i <= q_size - 2, else q_size - 1.  One block: chunk-level prefix, then element-level prefix
// inside the crossing chunk.
template <class Acc>
__global__ void __launch_bounds__(kScanThreads) search_kernel(const double2* __restrict__ psi, uint64_t q_size,
                                                               const double* __restrict__ pchunk,
                                                               const double* __restrict__ d_inv, double u01,
                                                               uint64_t* __restrict__ d_idx) {
    __shared__ double sm[32];
    __shared__ double s_incl[kScanThreads];
    __shared__ unsigned long long s_found;
    __shared__ double s_before;
    __shared__ double s_chosen;
    const int t = threadIdx.x;
    const uint64_t nq = (q_size + kChunk - 1) / kChunk;
    const uint64_t per = (nq + kScanThreads - 1) / kScanThreads;
    const uint64_t c0 = (uint64_t)t * per;
    double local = 0.0;
    for (uint64_t c = c0; c < c0 + per && c < nq; ++c) local += pchunk[c];
    double total;
    const double incl = block_inclusive_scan<kScanThreads>(local, sm, &total);
    s_incl[t] = incl;
    if (t == 0) {
        s_found = ~0ull;
        s_chosen = u01 * total;
    }
    __syncthreads();
    const double chosen = s_chosen;
    const double excl = t ? s_incl[t - 1] : 0.0;
    // The first thread whose range crosses `chosen` scans its chunks.
    if (incl > chosen && !(excl > chosen)) {
        double run = excl;
        for (uint64_t c = c0; c < c0 + per && c < nq; ++c) {
            const double nxt = run + pchunk[c];
            if (nxt > chosen) {
                s_found = (unsigned long long)c;
                s_before = run;
                break;
            }
            run = nxt;
        }
    }
    __syncthreads();
    const unsigned long long chunk = s_found;
    if (chunk == ~0ull) {
        if (t == 0) *d_idx = q_size - 1;
        return;
    }
    const double before = s_before;
    const double inv = *d_inv;
    // Element level: thread t owns kChunk / kScanThreads contiguous amplitudes of the chunk.
    constexpr int per_t = (int)(kChunk / kScanThreads);
    const uint64_t e0 = (uint64_t)chunk * kChunk + (uint64_t)t * per_t;
    double p[per_t];
    double ls = 0.0;
#pragma unroll
    for (int k = 0; k < per_t; ++k) {
        const uint64_t i = e0 + k;
        p[k] = (i < q_size) ? nsq(Acc::load(psi, i)) * inv : 0.0;
        ls += p[k];
    }
    __syncthreads();
    double tot2;
    const double incl2 = block_inclusive_scan<kScanThreads>(ls, sm, &tot2);
    __syncthreads();
    s_incl[t] = incl2;
    if (t == 0) s_found = ~0ull;
    __syncthreads();
    double run = before + (t ? s_incl[t - 1] : 0.0);
#pragma unroll
    for (int k = 0; k < per_t; ++k) {
        run += p[k];
        const uint64_t i = e0 + k;
        if (i < q_size && run > chosen) {
            atomicMin(&s_found, (unsigned long long)i);
            break;
        }
    }
    __syncthreads();
    if (t == 0) {
        unsigned long long f = s_found;
        if (f == ~0ull) {
            // The chunk total and its element prefix differ by rounding only: take the chunk's last
            // index (the boundary lies within an ulp of `chosen`).
            uint64_t last = (uint64_t)chunk * kChunk + kChunk - 1;
            f = last < q_size ? last : q_size - 1;
        }
        if (f > q_size - 2) f = q_size - 1;  // cumulative_weights has q_size - 1 entries
        *d_idx = f;
    }
}

template <class Acc>
__global__ void collapse_kernel(double2* __restrict__ psi, uint64_t len, const uint64_t* __restrict__ d_idx,
                                uint64_t mask) {
    const uint64_t idy = *d_idx;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += stride)
        if (((i ^ idy) & mask) != 0) Acc::store(psi, i, make_double2(0.0, 0.0));
}

template <class Acc>
__global__ void scale_kernel(double2* __restrict__ psi, uint64_t len, const double* __restrict__ d_abs, int mode) {
    // mode 0: qvnt `normalize` thresholds (quant.rs:397-414); mode 1: always rescale to unit norm.
    const double norm = sqrt(*d_abs);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    if (norm <= 1e-15) {
        if (mode == 1) return;
        for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += stride)
            Acc::store(psi, i, make_double2(i == 0 ? 1.0 : 0.0, 0.0));
        return;
    }
    if (mode == 0 && 1. - norm <= 1e-9) return;
    const double inv = 1. / norm;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += stride) {
        double2 v = Acc::load(psi, i);
        Acc::store(psi, i, make_double2(v.x * inv, v.y * inv));
    }
}

template <class Acc>
__global__ void prob_kernel(const double2* __restrict__ psi, uint64_t first, uint64_t count,
                            const double* __restrict__ d_inv, double* __restrict__ out) {
    const double inv = *d_inv;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += stride)
        out[k] = nsq(Acc::load(psi, first + k)) * inv;
}

template <class Acc>
__global__ void polar_kernel(const double2* __restrict__ psi, uint64_t first, uint64_t count, double* __restrict__ out) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += stride) {
        double2 v = Acc::load(psi, first + k);
        out[2 * k] = hypot(v.x, v.y);
        out[2 * k + 1] = atan2(v.y, v.x);
    }
}

template <class Acc>
__global__ void copy_out_kernel(const double2* __restrict__ psi, uint64_t first, uint64_t count,
                                double2* __restrict__ out) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += stride)
        out[k] = Acc::load(psi, first + k);
}

template <class Acc>
__global__ void copy_in_kernel(double2* __restrict__ psi, uint64_t first, uint64_t count,
                               const double2* __restrict__ in) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += stride)
        Acc::store(psi, first + k, in[k]);
}

template <class Acc>
__global__ void reset_kernel(double2* __restrict__ psi, uint64_t len, uint64_t state) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += stride)
        Acc::store(psi, i, make_double2(i == state ? 1.0 : 0.0, 0.0));
}

template <class Acc>
__global__ void zero_mask_kernel(double2* __restrict__ psi, uint64_t len, uint64_t mask) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += stride)
        if (i & mask) Acc::store(psi, i, make_double2(0.0, 0.0));
}

template <class AccA, class AccB, class AccO>
__global__ void tensor_kernel(const double2* __restrict__ a, uint32_t na, const double2* __restrict__ b, uint32_t nb,
                              double2* __restrict__ out, uint64_t out_len) {
    const uint64_t q_size = 1ull << (na + nb);
    const uint64_t ma = (1ull << na) - 1, mb = (1ull << nb) - 1;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < out_len; i += stride)
        AccO::store(out, i, i < q_size ? c_mul(AccA::load(a, i & ma), AccB::load(b, (i >> na) & mb))
                                       : make_double2(0.0, 0.0));
}

template <class AccS, class AccD>
__global__ void convert_fmt_kernel(const double2* __restrict__ src, double2* __restrict__ dst, uint64_t len) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += stride)
        AccD::store(dst, i, AccS::load(src, i));
}

template <class Acc>
__global__ void rescale_kernel(double2* __restrict__ psi, uint64_t len, const double* __restrict__ d_target,
                               const double* __restrict__ d_current) {
    const double tgt = *d_target, cur = *d_current;
    if (!(tgt > 0.0) || !(cur > 0.0)) return;
    const double f = sqrt(tgt / cur);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += stride) {
        const double2 v = Acc::load(psi, i);
        Acc::store(psi, i, make_double2(v.x * f, v.y * f));
    }
}

// Chunk partials of <a|b> = sum conj(a_i) b_i, |a|^2, |b|^2 and max |a_i - b_i|.
template <class AccA, class AccB>
__global__ void __launch_bounds__(kRedThreads) overlap_chunk_kernel(const double2* __restrict__ a,
                                                                     const double2* __restrict__ b, uint64_t len,
                                                                     double* __restrict__ part) {
    __shared__ double sm[32];
    const uint64_t base = (uint64_t)blockIdx.x * kChunk;
    const uint64_t nc = gridDim.x;
    double re = 0.0, im = 0.0, na = 0.0, nb = 0.0, mx = 0.0;
    for (uint32_t k = threadIdx.x; k < kChunk; k += kRedThreads) {
        const uint64_t i = base + k;
        if (i >= len) break;
        const double2 x = AccA::load(a, i), y = AccB::load(b, i);
        re += x.x * y.x + x.y * y.y;
        im += x.x * y.y - x.y * y.x;
        na += nsq(x);
        nb += nsq(y);
        mx = fmax(mx, hypot(x.x - y.x, x.y - y.y));
    }
    const double r0 = block_sum<kRedThreads>(re, sm);
    const double r1 = block_sum<kRedThreads>(im, sm);
    const double r2 = block_sum<kRedThreads>(na, sm);
    const double r3 = block_sum<kRedThreads>(nb, sm);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (int w = 0; w < kRedThreads / 32; ++w) m = fmax(m, sm[w]);
        part[blockIdx.x] = r0;
        part[nc + blockIdx.x] = r1;
        part[2 * nc + blockIdx.x] = r2;
        part[3 * nc + blockIdx.x] = r3;
        part[4 * nc + blockIdx.x] = m;
    }
}

__global__ void __launch_bounds__(kScanThreads) overlap_final_kernel(const double* __restrict__ part, uint64_t nc,
                                                                      double* __restrict__ out) {
    __shared__ double sm[32];
    for (int q = 0; q < 4; ++q) {
        double s = 0.0;
        for (uint64_t k = threadIdx.x; k < nc; k += kScanThreads) s += part[q * nc + k];
        const double t = block_sum<kScanThreads>(s, sm);
        if (threadIdx.x == 0) out[q] = t;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (uint64_t k = 0; k < nc; ++k) m = fmax(m, part[4 * nc + k]);
        out[4] = m;
    }
}

// Standard normal draw for sample_all when the caller injects none: two uniforms from SplitMix64 of
// (seed, index), Box-Muller with the device's log / sqrt / cospi.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double std_normal(uint64_t seed, uint64_t i) {
    const uint64_t a = mix64(seed ^ (2 * i)), b = mix64(seed ^ (2 * i + 1));
    const double u1 = ((double)(a >> 11) + 1.0) * (1.0 / 9007199254740992.0);  // (0, 1]
    const double u2 = (double)(b >> 11) * (1.0 / 9007199254740992.0);          // [0, 1)
    return sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
}

// sample_all, step 1 (quant.rs:513-535): n_i = sqrt(p_i) z_i with p_i = |psi_i|^2 * inv, into n[];
// chunk partial sums of n for n_sum.
template <class Acc>
__global__ void __launch_bounds__(kRedThreads) sample_noise_kernel(const double2* __restrict__ psi, uint64_t q_size,
                                                                    const double* __restrict__ d_inv,
                                                                    const double* __restrict__ z, uint64_t seed,
                                                                    double* __restrict__ n, double* __restrict__ part) {
    __shared__ double sm[32];
    const double inv = *d_inv;
    const uint64_t base = (uint64_t)blockIdx.x * kChunk;
    double s = 0.0;
    for (uint32_t k = threadIdx.x; k < kChunk; k += kRedThreads) {
        const uint64_t i = base + k;
        if (i >= q_size) break;
        const double p = nsq(Acc::load(psi, i)) * inv;
        const double v = sqrt(p) * (z ? z[i] : std_normal(seed, i));
        n[i] = v;
        s += v;
    }
    const double t = block_sum<kRedThreads>(s, sm);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// sample_all, step 2 (quant.rs:537-543): counts (c p_i + sqrt(c) (n_i - n_sum p_i)).round().max(0),
// written over n[] as int64.
template <class Acc>
__global__ void sample_count_kernel(const double2* __restrict__ psi, uint64_t q_size, const double* __restrict__ d_inv,
                                    const double* __restrict__ d_nsum, double c, double* __restrict__ n) {
    const double inv = *d_inv, n_sum = *d_nsum, c_sqrt = sqrt(c);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < q_size; i += stride) {
        const double p = nsq(Acc::load(psi, i)) * inv;
        const double v = round(c * p + c_sqrt * (n[i] - n_sum * p));
        const long long k = isnan(v) ? 0 : (long long)v;
        reinterpret_cast<long long*>(n)[i] = k > 0 ? k : 0;
    }
}

// combine_with_unitary (quant.rs:273-308) and linear_composition (quant.rs:311-328).
template <class AccA, class AccB, class AccO>
__global__ void combine_kernel(const double2* __restrict__ a, const double2* __restrict__ b, uint64_t q_mask,
                               double2 c00, double2 c01, double2 c10, double2 c11, double2* __restrict__ out,
                               uint64_t out_len) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < out_len; i += stride) {
        const double2 qa = AccA::load(a, q_mask & i), qb = AccB::load(b, q_mask & i);
        const bool low = (~q_mask & i) == 0;
        AccO::store(out, i, low ? c_add(c_mul(c00, qa), c_mul(c01, qb)) : c_add(c_mul(c10, qa), c_mul(c11, qb)));
    }
}

template <class Acc, class AccP>
__global__ void linear_kernel(double2* __restrict__ self, const double2* __restrict__ psi, uint64_t len, double2 c0,
                              double2 c1) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += stride)
        Acc::store(self, i, c_add(c_mul(Acc::load(self, i), c0), c_mul(AccP::load(psi, i), c1)));
}

// Storage conversion in place: f64 -> df64 (to_df = 1) or df64 -> f64 (to_df = 0).
__global__ void convert_kernel(double2* __restrict__ psi, uint64_t len, int to_df) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += stride) {
        if (to_df) {
            const double2 v = psi[i];
            AccDF64::store(psi, i, v);
        } else {
            psi[i] = AccDF64::load(psi, i);
        }
    }
}

unsigned flat_grid(uint64_t n) {
    uint64_t g = (n + 255) / 256;
    const uint64_t cap = 152ull * 16;
    if (g > cap) g = cap;
    return (unsigned)(g < 1 ? 1 : g);
}

#define QVNT_BY_FMT(fmt, KERNEL, ...)                          \
    do {                                                       \
        if ((fmt) == FMT_DF64) KERNEL<AccDF64> __VA_ARGS__;    \
        else if ((fmt) == FMT_C32) KERNEL<AccC32> __VA_ARGS__; \
        else KERNEL<AccF64> __VA_ARGS__;                       \
    } while (0)

}  // namespace

int launch_norm_sqr_sum(const double2* psi, int fmt, uint64_t len, double* scratch, double* d_out, cudaStream_t stream) {
    const uint64_t nc = chunk_count(len);
    QVNT_BY_FMT(fmt, chunk_sum_kernel, <<<(unsigned)nc, kRedThreads, 0, stream>>>(psi, len, nullptr, scratch));
    final_sum_kernel<<<1, kScanThreads, 0, stream>>>(scratch, nc, d_out);
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

int launch_measure(double2* psi, int fmt, uint64_t len, uint64_t q_size, uint64_t mask, double u01, double* scratch,
                   uint64_t* d_idx, int* d_status, int renormalise, cudaStream_t stream) {
    const uint64_t nc = chunk_count(len);
    double* partial = scratch;
    double* pchunk = scratch + nc;
    double* d_abs = scratch + 2 * nc;
    double* d_inv = d_abs + 1;
    QVNT_BY_FMT(fmt, chunk_sum_kernel, <<<(unsigned)nc, kRedThreads, 0, stream>>>(psi, len, nullptr, partial));
    final_sum_kernel<<<1, kScanThreads, 0, stream>>>(partial, nc, d_abs);
    inv_kernel<<<1, 1, 0, stream>>>(d_abs, d_inv, d_status);
    QVNT_BY_FMT(fmt, chunk_sum_kernel,
                <<<(unsigned)chunk_count(q_size), kRedThreads, 0, stream>>>(psi, q_size, d_inv, pchunk));
    QVNT_BY_FMT(fmt, search_kernel, <<<1, kScanThreads, 0, stream>>>(psi, q_size, pchunk, d_inv, u01, d_idx));
    QVNT_BY_FMT(fmt, collapse_kernel, <<<flat_grid(len), 256, 0, stream>>>(psi, len, d_idx, mask));
    if (renormalise) {
        QVNT_BY_FMT(fmt, chunk_sum_kernel, <<<(unsigned)nc, kRedThreads, 0, stream>>>(psi, len, nullptr, partial));
        final_sum_kernel<<<1, kScanThreads, 0, stream>>>(partial, nc, d_abs);
        QVNT_BY_FMT(fmt, scale_kernel, <<<flat_grid(len), 256, 0, stream>>>(psi, len, d_abs, 1));
    }
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

int launch_inv(const double* d_abs, double* d_inv, int* d_status, cudaStream_t stream) {
    inv_kernel<<<1, 1, 0, stream>>>(d_abs, d_inv, d_status);
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

int launch_probabilities(const double2* psi, int fmt, uint64_t first, uint64_t count, const double* d_inv_abs,
                         double* d_out, cudaStream_t stream) {
    QVNT_BY_FMT(fmt, prob_kernel, <<<flat_grid(count), 256, 0, stream>>>(psi, first, count, d_inv_abs, d_out));
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

int launch_polar(const double2* psi, int fmt, uint64_t first, uint64_t count, double* d_out, cudaStream_t stream) {
    QVNT_BY_FMT(fmt, polar_kernel, <<<flat_grid(count), 256, 0, stream>>>(psi, first, count, d_out));
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

int launch_copy_out(const double2* psi, int fmt, uint64_t first, uint64_t count, double2* d_out, cudaStream_t stream) {
    QVNT_BY_FMT(fmt, copy_out_kernel, <<<flat_grid(count), 256, 0, stream>>>(psi, first, count, d_out));
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

int launch_copy_in(double2* psi, int fmt, uint64_t first, uint64_t count, const double2* d_in, cudaStream_t stream) {
    QVNT_BY_FMT(fmt, copy_in_kernel, <<<flat_grid(count), 256, 0, stream>>>(psi, first, count, d_in));
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

int launch_reset(double2* psi, int fmt, uint64_t len, uint64_t state, cudaStream_t stream) {
    QVNT_BY_FMT(fmt, reset_kernel, <<<flat_grid(len), 256, 0, stream>>>(psi, len, state));
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

int launch_zero_mask(double2* psi, int fmt, uint64_t len, uint64_t mask, cudaStream_t stream) {
    QVNT_BY_FMT(fmt, zero_mask_kernel, <<<flat_grid(len), 256, 0, stream>>>(psi, len, mask));
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

int launch_normalize(double2* psi, int fmt, uint64_t len, const double* d_abs, cudaStream_t stream) {
    QVNT_BY_FMT(fmt, scale_kernel, <<<flat_grid(len), 256, 0, stream>>>(psi, len, d_abs, 0));
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

int launch_tensor(const double2* a, int fa, uint32_t na, const double2* b, int fb, uint32_t nb, double2* out, int fo,
                  uint64_t out_len, cudaStream_t stream) {
    const unsigned g = flat_grid(out_len);
    const int code = (fa << 2) | (fb << 1) | fo;
    switch (code) {
    case 0: tensor_kernel<AccF64, AccF64, AccF64><<<g, 256, 0, stream>>>(a, na, b, nb, out, out_len); break;
    case 1: tensor_kernel<AccF64, AccF64, AccDF64><<<g, 256, 0, stream>>>(a, na, b, nb, out, out_len); break;
    case 2: tensor_kernel<AccF64, AccDF64, AccF64><<<g, 256, 0, stream>>>(a, na, b, nb, out, out_len); break;
    case 3: tensor_kernel<AccF64, AccDF64, AccDF64><<<g, 256, 0, stream>>>(a, na, b, nb, out, out_len); break;
    case 4: tensor_kernel<AccDF64, AccF64, AccF64><<<g, 256, 0, stream>>>(a, na, b, nb, out, out_len); break;
    case 5: tensor_kernel<AccDF64, AccF64, AccDF64><<<g, 256, 0, stream>>>(a, na, b, nb, out, out_len); break;
    case 6: tensor_kernel<AccDF64, AccDF64, AccF64><<<g, 256, 0, stream>>>(a, na, b, nb, out, out_len); break;
    default: tensor_kernel<AccDF64, AccDF64, AccDF64><<<g, 256, 0, stream>>>(a, na, b, nb, out, out_len); break;
    }
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

int launch_convert(double2* psi, uint64_t len, int to_df, cudaStream_t stream) {
    convert_kernel<<<flat_grid(len), 256, 0, stream>>>(psi, len, to_df);
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

namespace {
template <class AccS>
void convert_from(const double2* src, double2* dst, int fdst, uint64_t len, cudaStream_t stream) {
    const unsigned g = flat_grid(len);
    if (fdst == FMT_DF64) convert_fmt_kernel<AccS, AccDF64><<<g, 256, 0, stream>>>(src, dst, len);
    else if (fdst == FMT_C32) convert_fmt_kernel<AccS, AccC32><<<g, 256, 0, stream>>>(src, dst, len);
    else convert_fmt_kernel<AccS, AccF64><<<g, 256, 0, stream>>>(src, dst, len);
}

template <class AccA>
void overlap_with(const double2* a, const double2* b, int fb, uint64_t len, double* part, cudaStream_t stream) {
    const unsigned nc = (unsigned)chunk_count(len);
    if (fb == FMT_DF64) overlap_chunk_kernel<AccA, AccDF64><<<nc, kRedThreads, 0, stream>>>(a, b, len, part);
    else if (fb == FMT_C32) overlap_chunk_kernel<AccA, AccC32><<<nc, kRedThreads, 0, stream>>>(a, b, len, part);
    else overlap_chunk_kernel<AccA, AccF64><<<nc, kRedThreads, 0, stream>>>(a, b, len, part);
}
}  // namespace

int launch_sample_all(const double2* psi, int fmt, uint64_t q_size, const double* d_inv, const double* d_z,
                      uint64_t seed, uint64_t count, double* d_n, double* scratch, double* d_nsum,
                      cudaStream_t stream) {
    const uint64_t nc = chunk_count(q_size);
    QVNT_BY_FMT(fmt, sample_noise_kernel,
                <<<(unsigned)nc, kRedThreads, 0, stream>>>(psi, q_size, d_inv, d_z, seed, d_n, scratch));
    final_sum_kernel<<<1, kScanThreads, 0, stream>>>(scratch, nc, d_nsum);
    QVNT_BY_FMT(fmt, sample_count_kernel,
                <<<flat_grid(q_size), 256, 0, stream>>>(psi, q_size, d_inv, d_nsum, (double)count, d_n));
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

int launch_combine(const double2* a, int fa, const double2* b, int fb, uint32_t n, const double* c, double2* out,
                   int fo, uint64_t out_len, cudaStream_t stream) {
    const uint64_t q_mask = (1ull << n) - 1;
    const double2 c00 = make_double2(c[0], c[1]), c01 = make_double2(c[2], c[3]);
    const double2 c10 = make_double2(c[4], c[5]), c11 = make_double2(c[6], c[7]);
    const unsigned g = flat_grid(out_len);
    const int code = (fa << 2) | (fb << 1) | fo;
#define QVNT_COMBINE(A, B, O) combine_kernel<A, B, O><<<g, 256, 0, stream>>>(a, b, q_mask, c00, c01, c10, c11, out, out_len)
    switch (code) {
    case 0: QVNT_COMBINE(AccF64, AccF64, AccF64); break;
    case 1: QVNT_COMBINE(AccF64, AccF64, AccDF64); break;
    case 2: QVNT_COMBINE(AccF64, AccDF64, AccF64); break;
    case 3: QVNT_COMBINE(AccF64, AccDF64, AccDF64); break;
    case 4: QVNT_COMBINE(AccDF64, AccF64, AccF64); break;
    case 5: QVNT_COMBINE(AccDF64, AccF64, AccDF64); break;
    case 6: QVNT_COMBINE(AccDF64, AccDF64, AccF64); break;
    default: QVNT_COMBINE(AccDF64, AccDF64, AccDF64); break;
    }
#undef QVNT_COMBINE
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

int launch_linear(double2* self, int fs, const double2* psi, int fp, uint64_t len, const double* c,
                  cudaStream_t stream) {
    const double2 c0 = make_double2(c[0], c[1]), c1 = make_double2(c[2], c[3]);
    const unsigned g = flat_grid(len);
    switch ((fs << 1) | fp) {
    case 0: linear_kernel<AccF64, AccF64><<<g, 256, 0, stream>>>(self, psi, len, c0, c1); break;
    case 1: linear_kernel<AccF64, AccDF64><<<g, 256, 0, stream>>>(self, psi, len, c0, c1); break;
    case 2: linear_kernel<AccDF64, AccF64><<<g, 256, 0, stream>>>(self, psi, len, c0, c1); break;
    default: linear_kernel<AccDF64, AccDF64><<<g, 256, 0, stream>>>(self, psi, len, c0, c1); break;
    }
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

int launch_convert_fmt(const double2* src, int fsrc, double2* dst, int fdst, uint64_t len, cudaStream_t stream) {
    if (fsrc == FMT_DF64) convert_from<AccDF64>(src, dst, fdst, len, stream);
    else if (fsrc == FMT_C32) convert_from<AccC32>(src, dst, fdst, len, stream);
    else convert_from<AccF64>(src, dst, fdst, len, stream);
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

int launch_rescale(double2* psi, int fmt, uint64_t len, const double* d_target, const double* d_current,
                   cudaStream_t stream) {
    QVNT_BY_FMT(fmt, rescale_kernel, <<<flat_grid(len), 256, 0, stream>>>(psi, len, d_target, d_current));
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

int launch_overlap(const double2* a, int fa, const double2* b, int fb, uint64_t len, double* scratch, double* d_out,
                   cudaStream_t stream) {
    if (fa == FMT_DF64) overlap_with<AccDF64>(a, b, fb, len, scratch, stream);
    else if (fa == FMT_C32) overlap_with<AccC32>(a, b, fb, len, scratch, stream);
    else overlap_with<AccF64>(a, b, fb, len, scratch, stream);
    overlap_final_kernel<<<1, kScanThreads, 0, stream>>>(scratch, chunk_count(len), d_out);
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

// ---- allocation-free norm: scratch in a file-scope device array ---------------------------------
// Chunk partial sums of qvnt_norm_sqr_noalloc.  Every GPU that loads the library holds this array
// (512 KiB) until the process exits; all calls on a device share it.
constexpr uint64_t kNoAllocPartials = QVNT_NOALLOC_MAX_AMPLITUDES / kChunk;
static __device__ __align__(256) double g_noalloc_partials[kNoAllocPartials];

namespace {
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[kNoAllocMaxDevices] = {};
}  // namespace

}  // namespace qvnt

using namespace qvnt;

// For callers that cannot allocate device memory themselves: the partial sums live in
// g_noalloc_partials.  Host code cannot use the array's name as a device address, so the address
// is looked up once per device (with that device current) and cached.
extern "C" int qvnt_norm_sqr_noalloc(const double* d_psi, uint64_t len, double* d_out, void* stream) {
    if (!d_psi || !d_out) return set_error(QVNT_ERR_BAD_ARG, "null device pointer");
    // the kernels read amplitudes as 16-byte double2 and write *d_out as a double: a misaligned
    // pointer would fault the caller's context, so it is refused here
    if (reinterpret_cast<uintptr_t>(d_psi) & 15u)
        return set_error(QVNT_ERR_BAD_ARG, "d_psi is not 16-byte aligned (amplitudes are read as double2)");
    if (reinterpret_cast<uintptr_t>(d_out) & 7u) return set_error(QVNT_ERR_BAD_ARG, "d_out is not 8-byte aligned");
    if (len == 0) return set_error(QVNT_ERR_BAD_ARG, "empty state");
    if (len > QVNT_NOALLOC_MAX_AMPLITUDES)
        return set_error(QVNT_ERR_BAD_ARG, "state of %llu amplitudes exceeds the allocation-free limit of %llu",
                         (unsigned long long)len, (unsigned long long)QVNT_NOALLOC_MAX_AMPLITUDES);
    int dev = 0;
    QVNT_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return set_error(QVNT_ERR_BAD_ARG, "device %d out of range", dev);
    double* partials = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
            if (e != cudaSuccess) return set_cuda_error(e, "cudaGetSymbolAddress(g_noalloc_partials)");
            g_noalloc_ptr[dev] = static_cast<double*>(p);
        }
        partials = g_noalloc_ptr[dev];
    }
    // Every chunk writes its own partial and the final block overwrites *d_out, so nothing left
    // in the array by an earlier call is read: no clearing is needed.
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint64_t nc = chunk_count(len);
    chunk_sum_kernel<AccF64><<<(unsigned)nc, kRedThreads, 0, s>>>(reinterpret_cast<const double2*>(d_psi), len,
                                                                   nullptr, partials);
    final_sum_kernel<<<1, kScanThreads, 0, s>>>(partials, nc, d_out);
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}
