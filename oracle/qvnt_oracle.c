/*
 * qvnt_oracle.c - CPU restatement of qvnt 0.4.4's state-vector arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU engine (see qvnt_oracle.h).  Compiled with
 * -ffp-contract=off and without fast-math so that each expression rounds exactly as qvnt's
 * release build does.  Paths below are relative to the qvnt crate root.
 */
#include "qvnt_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- num-complex 0.4 arithmetic (Add, Sub, Mul, Neg, scale) -------------------------------- */
static inline oc_t c_add(oc_t a, oc_t b) { oc_t r = {a.re + b.re, a.im + b.im}; return r; }
static inline oc_t c_neg(oc_t a) { oc_t r = {-a.re, -a.im}; return r; }
static inline oc_t c_mul(oc_t a, oc_t b) {
    oc_t r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}
static inline oc_t c_scale(oc_t a, double t) { oc_t r = {a.re * t, a.im * t}; return r; }
static inline oc_t c_conj(oc_t a) { oc_t r = {a.re, -a.im}; return r; }

static inline unsigned popc(uint64_t x) { return (unsigned)__builtin_popcountll(x); }

static const double FRAC_1_SQRT_2 = 0.70710678118654752440084436210484903;

/* `rotate(z, q)`: multiply by i^q (src/math/mod.rs:40-50). */
static inline oc_t rotate(oc_t z, uint64_t q) {
    if (q & 2) {
        z.re = -z.re;
        z.im = -z.im;
    }
    if (q & 1) {
        double t = -z.im; /* z.im = -z.im; swap(re, im) */
        z.im = z.re;
        z.re = t;
    }
    return z;
}

static inline oc_t gate_m(const qvnt_gate* g, int k) {
    oc_t r = {g->matrix[2 * k], g->matrix[2 * k + 1]};
    return r;
}

oc_t oracle_atomic(const qvnt_gate* g, const oc_t* psi, uint64_t idx) {
    const uint64_t a = g->a_mask;
    switch (g->kind) {
    case QVNT_GATE_ID: /* id.rs:7-9 */
        return psi[idx];
    case QVNT_GATE_X: /* x.rs:15-17 */
        return psi[idx ^ a];
    case QVNT_GATE_Y: { /* y.rs:10-13, :17-23 */
        uint64_t i_pow = (uint64_t)(uint32_t)(~(uint32_t)(popc(a) + 1u));
        if ((popc(idx & a) & 1u) == 0) i_pow ^= 2;
        return rotate(psi[idx ^ a], i_pow);
    }
    case QVNT_GATE_Z: /* z.rs:15-21 */
        return (popc(idx & a) & 1u) == 1 ? c_neg(psi[idx]) : psi[idx];
    case QVNT_GATE_S: { /* s.rs:19-25 */
        uint64_t count = popc(idx & a);
        if (g->dagger) count = (~count) + 1u;
        return rotate(psi[idx], count);
    }
    case QVNT_GATE_T: { /* t.rs:24-35 */
        const oc_t e = {FRAC_1_SQRT_2, FRAC_1_SQRT_2};
        uint64_t count = popc(idx & a);
        if (g->dagger) count = (~count) + 1u;
        oc_t p = rotate(psi[idx], count >> 1);
        return (count & 1u) == 1 ? c_mul(e, p) : p;
    }
    case QVNT_GATE_RX:   /* rx.rs:18-24 */
    case QVNT_GATE_RXX: { /* rxx.rs:19-25 (same formula over ab_mask) */
        oc_t p0 = psi[idx], p1 = psi[idx ^ a];
        oc_t r = {p0.re * g->phase[0] + p1.im * g->phase[1], p0.im * g->phase[0] - p1.re * g->phase[1]};
        return r;
    }
    case QVNT_GATE_RY: { /* ry.rs:19-29 */
        double pr = g->phase[0], pi = g->phase[1];
        oc_t p0 = psi[idx], p1 = psi[idx ^ a];
        if ((idx & a) == 0) pi = -pi;
        oc_t r = {p0.re * pr + p1.re * pi, p0.im * pr + p1.im * pi};
        return r;
    }
    case QVNT_GATE_RYY: { /* ryy.rs:19-29 */
        double pr = g->phase[0], pi = g->phase[1];
        oc_t p0 = psi[idx], p1 = psi[idx ^ a];
        if ((popc(idx & a) & 1u) == 0) pi = -pi;
        oc_t r = {p0.re * pr + p1.im * pi, p0.im * pr - p1.re * pi};
        return r;
    }
    case QVNT_GATE_RZ: { /* rz.rs:19-25 */
        oc_t ph = {g->phase[0], g->phase[1]};
        if ((idx & a) == 0) ph.im = -ph.im;
        return c_mul(ph, psi[idx]);
    }
    case QVNT_GATE_RZZ: { /* rzz.rs:19-25 */
        oc_t ph = {g->phase[0], g->phase[1]};
        if ((popc(idx & a) & 1u) == 0) ph.im = -ph.im;
        return c_mul(ph, psi[idx]);
    }
    case QVNT_GATE_U1: { /* u1.rs:17-25 */
        int a_bit = (idx & a) != 0;
        uint64_t i = idx & ~a;
        if (!a_bit) return c_add(c_mul(gate_m(g, 0), psi[i]), c_mul(gate_m(g, 1), psi[i | a]));
        return c_add(c_mul(gate_m(g, 2), psi[i]), c_mul(gate_m(g, 3), psi[i | a]));
    }
    case QVNT_GATE_U2: { /* u2.rs:22-49 */
        const uint64_t b = g->b_mask;
        int a_bit = (idx & a) != 0, b_bit = (idx & b) != 0;
        uint64_t i = idx & ~a & ~b;
        int row = (b_bit << 1) | a_bit;
        oc_t s = c_mul(gate_m(g, 4 * row + 0), psi[i]);
        s = c_add(s, c_mul(gate_m(g, 4 * row + 1), psi[i | a]));
        s = c_add(s, c_mul(gate_m(g, 4 * row + 2), psi[i | b]));
        s = c_add(s, c_mul(gate_m(g, 4 * row + 3), psi[i | a | b]));
        return s;
    }
    case QVNT_GATE_H1: { /* h1.rs:16-22 */
        oc_t p0 = psi[idx], p1 = psi[idx ^ a];
        if (idx & a) p0 = c_neg(p0);
        return c_scale(c_add(p0, p1), FRAC_1_SQRT_2);
    }
    case QVNT_GATE_H2: { /* h2.rs:22-38 */
        const uint64_t b = g->b_mask, ab = a | b;
        oc_t p0 = psi[idx], p1 = psi[idx ^ a], p2 = psi[idx ^ b], p3 = psi[idx ^ ab];
        if (idx & a) {
            p0 = c_neg(p0);
            p2 = c_neg(p2);
        }
        if (idx & b) {
            p0 = c_neg(p0);
            p1 = c_neg(p1);
        }
        return c_scale(c_add(c_add(c_add(p0, p1), p2), p3), 0.5);
    }
    case QVNT_GATE_SWAP: /* swap.rs:16-22 */
        return (popc(idx & a) & 1u) == 1 ? psi[idx ^ a] : psi[idx];
    case QVNT_GATE_ISWAP: { /* i_swap.rs:20-37 */
        if ((popc(idx & a) & 1u) == 1) {
            oc_t p = psi[idx ^ a];
            oc_t r;
            if (g->dagger) { r.re = p.im; r.im = -p.re; }
            else { r.re = -p.im; r.im = p.re; }
            return r;
        }
        return psi[idx];
    }
    case QVNT_GATE_SQRT_SWAP: { /* sqrt_swap.rs:20-37 */
        if ((popc(idx & a) & 1u) == 1) {
            oc_t p0 = psi[idx], p1 = psi[idx ^ a];
            oc_t r;
            if (g->dagger) {
                r.re = 0.5 * (p0.re + p0.im + p1.re - p1.im);
                r.im = 0.5 * (p0.im - p0.re + p1.im + p1.re);
            } else {
                r.re = 0.5 * (p0.re - p0.im + p1.re + p1.im);
                r.im = 0.5 * (p0.im + p0.re + p1.im - p1.re);
            }
            return r;
        }
        return psi[idx];
    }
    case QVNT_GATE_SQRT_ISWAP: { /* sqrt_i_swap.rs:20-37 */
        if ((popc(idx & a) & 1u) == 1) {
            oc_t p0 = psi[idx], p1 = psi[idx ^ a];
            oc_t r;
            if (g->dagger) {
                r.re = FRAC_1_SQRT_2 * (p0.re + p1.im);
                r.im = FRAC_1_SQRT_2 * (p0.im - p1.re);
            } else {
                r.re = FRAC_1_SQRT_2 * (p0.re - p1.im);
                r.im = FRAC_1_SQRT_2 * (p0.im + p1.re);
            }
            return r;
        }
        return psi[idx];
    }
    default:
        return psi[idx];
    }
}

uint64_t oracle_acts_on(const qvnt_gate* g) {
    switch (g->kind) {
    case QVNT_GATE_ID: return 0;                          /* id.rs:15-17 */
    case QVNT_GATE_H2: return g->a_mask | g->b_mask;      /* h2.rs:50-52 (ab_mask) */
    case QVNT_GATE_U2: return g->a_mask;                  /* u2.rs:70-72: b_mask omitted */
    default: return g->a_mask;
    }
}

void oracle_for_each(const qvnt_gate* g, const oc_t* psi_i, oc_t* psi_o, uint64_t len, int nthreads) {
    const uint64_t ctrl = g->ctrl;
    int64_t n = (int64_t)len;
    (void)nthreads;
    if (ctrl != 0) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads) if (nthreads > 1)
#endif
        for (int64_t s = 0; s < n; ++s) {
            uint64_t idx = (uint64_t)s;
            psi_o[idx] = ((~idx & ctrl) == 0) ? oracle_atomic(g, psi_i, idx) : psi_i[idx];
        }
    } else {
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads) if (nthreads > 1)
#endif
        for (int64_t s = 0; s < n; ++s) psi_o[s] = oracle_atomic(g, psi_i, (uint64_t)s);
    }
}

void oracle_apply(const qvnt_gate* gates, size_t count, oc_t* psi, oc_t* scratch, uint64_t len,
                  int nthreads) {
    oc_t* cur = psi;
    oc_t* nxt = scratch;
    for (size_t k = 0; k < count; ++k) {
        oracle_for_each(&gates[k], cur, nxt, len, nthreads);
        oc_t* t = cur;
        cur = nxt;
        nxt = t;
    }
    if (cur != psi) memcpy(psi, cur, (size_t)len * sizeof(oc_t));
}

/* ---- registers (src/register/quant.rs) ---------------------------------------------------- */
uint64_t oracle_reg_len(uint32_t q_num) {
    uint64_t q_size = 1ull << q_num;
    return q_size < 8 ? 8 : q_size; /* MIN_BUFFER_LEN = 8 (:15) */
}

void oracle_reg_init(uint32_t q_num, uint64_t state, oc_t* psi) {
    uint64_t len = oracle_reg_len(q_num);
    uint64_t q_mask = (1ull << q_num) - 1;
    memset(psi, 0, (size_t)len * sizeof(oc_t));
    psi[state & q_mask].re = 1.0;
}

/* `norm_sqr` = re*re + im*im (num-complex) summed left to right from 0 (Single model). */
double oracle_get_absolute(const oc_t* psi, uint64_t len) {
    double s = 0.0;
    for (uint64_t i = 0; i < len; ++i) s += psi[i].re * psi[i].re + psi[i].im * psi[i].im;
    return s;
}

void oracle_get_probabilities(const oc_t* psi, uint64_t len, uint32_t q_num, double* out) {
    double abs_ = oracle_get_absolute(psi, len);
    double inv = 1. / abs_;
    uint64_t q_size = 1ull << q_num;
    for (uint64_t i = 0; i < q_size; ++i) out[i] = (psi[i].re * psi[i].re + psi[i].im * psi[i].im) * inv;
}

/* rand 0.8.5 `WeightedIndex::new` keeps cumulative_weights[j] = w_0 + ... + w_j for j < count-1
 * and total_weight = the sum of all; `sample` draws chosen in [0, total) and returns
 * `cumulative_weights.partition_point(|w| w <= chosen)`.  The draw is chosen = u01 * total. */
uint64_t oracle_weighted_index(const double* w, uint64_t count, double u01) {
    double total = w[0];
    for (uint64_t j = 1; j < count; ++j) total += w[j];
    double chosen = u01 * total;
    double run = w[0];
    for (uint64_t j = 0; j + 1 < count; ++j) {
        if (run > chosen) return j;
        run += w[j + 1];
    }
    return count - 1;
}

void oracle_collapse_mask(oc_t* psi, uint64_t len, uint64_t idy, uint64_t mask) {
    for (uint64_t idx = 0; idx < len; ++idx)
        if (((idx ^ idy) & mask) != 0) {
            psi[idx].re = 0.0;
            psi[idx].im = 0.0;
        }
}

uint64_t oracle_measure_mask(oc_t* psi, uint64_t len, uint32_t q_num, uint64_t mask, double u01,
                             uint64_t* chosen_idx) {
    uint64_t q_mask = (1ull << q_num) - 1;
    mask &= q_mask;
    if (mask == 0) {
        if (chosen_idx) *chosen_idx = 0;
        return 0;
    }
    uint64_t q_size = 1ull << q_num;
    double* p = (double*)malloc((size_t)q_size * sizeof(double));
    oracle_get_probabilities(psi, len, q_num, p);
    uint64_t idx = oracle_weighted_index(p, q_size, u01);
    free(p);
    oracle_collapse_mask(psi, len, idx, mask);
    if (chosen_idx) *chosen_idx = idx;
    return idx & mask;
}

void oracle_reset(oc_t* psi, uint64_t len, uint32_t q_num, uint64_t state) {
    uint64_t q_mask = (1ull << q_num) - 1;
    memset(psi, 0, (size_t)len * sizeof(oc_t));
    psi[q_mask & state].re = 1.0;
}

void oracle_normalize(oc_t* psi, uint64_t len, uint32_t q_num) {
    double norm = sqrt(oracle_get_absolute(psi, len));
    if (norm <= 1e-15) {
        oracle_reset(psi, len, q_num, 0);
        return;
    } else if (1. - norm <= 1e-9) {
        return;
    }
    norm = 1. / norm;
    for (uint64_t i = 0; i < len; ++i) {
        psi[i].re *= norm;
        psi[i].im *= norm;
    }
}

void oracle_reset_by_mask(oc_t* psi, uint64_t len, uint32_t q_num, uint64_t mask) {
    uint64_t q_mask = (1ull << q_num) - 1;
    if ((mask & q_mask) == q_mask) {
        oracle_reset(psi, len, q_num, 0);
        return;
    }
    for (uint64_t idx = 0; idx < len; ++idx)
        if ((idx & mask) != 0) {
            psi[idx].re = 0.0;
            psi[idx].im = 0.0;
        }
    oracle_normalize(psi, len, q_num);
}

void oracle_get_polar(const oc_t* psi, uint32_t q_num, double* out) {
    uint64_t q_size = 1ull << q_num;
    for (uint64_t i = 0; i < q_size; ++i) {
        out[2 * i] = hypot(psi[i].re, psi[i].im);   /* Complex::norm */
        out[2 * i + 1] = atan2(psi[i].im, psi[i].re); /* Complex::arg */
    }
}

void oracle_tensor(const oc_t* a, uint32_t na, const oc_t* b, uint32_t nb, oc_t* out) {
    uint32_t q_num = na + nb;
    uint64_t q_size = 1ull << q_num;
    uint64_t len = oracle_reg_len(q_num);
    uint64_t ma = (1ull << na) - 1, mb = (1ull << nb) - 1;
    for (uint64_t idx = 0; idx < len; ++idx) {
        if (idx < q_size) out[idx] = c_mul(a[idx & ma], b[(idx >> na) & mb]);
        else { out[idx].re = 0.0; out[idx].im = 0.0; }
    }
}

/* src/register/quant.rs:513-594.  p = get_probabilities(); n_i = sqrt(p_i) * z_i; n_sum = the
 * sequential sum; counts (p_i c + sqrt(c) (n_i - n_sum p_i)).round().max(0); then the total is
 * corrected to `count`: a deficit adds (delta >> q_num) to every entry and one more to the first
 * (delta % q_mask) entries (q_mask, not q_size, as written there); an excess removes one at a time
 * from the first nonzero entries of idx & q_mask, idx = 0, 1, ... */
int oracle_sample_all(const oc_t* psi, uint64_t len, uint32_t q_num, uint64_t count, const double* z,
                      uint64_t* out) {
    const uint64_t q_size = 1ull << q_num, q_mask = q_size - 1;
    if (len != q_size || q_mask == 0) return -1;
    double* p = (double*)malloc(q_size * sizeof(double));
    double* n = (double*)malloc(q_size * sizeof(double));
    oracle_get_probabilities(psi, len, q_num, p);
    const double c = (double)count;
    const double c_sqrt = sqrt(c);
    for (uint64_t i = 0; i < q_size; ++i) n[i] = sqrt(p[i]) * z[i];
    double n_sum = 0.0;
    for (uint64_t i = 0; i < q_size; ++i) n_sum += n[i];
    int64_t total = 0;
    for (uint64_t i = 0; i < q_size; ++i) {
        double v = round(c * p[i] + c_sqrt * (n[i] - n_sum * p[i]));
        int64_t k = v != v ? 0 : (int64_t)v;  /* Rust `as` maps NaN to 0 */
        out[i] = (uint64_t)(k > 0 ? k : 0);
        total += (int64_t)out[i];
    }
    int64_t delta = total - (int64_t)count;
    if (delta < 0) {
        const uint64_t d = (uint64_t)(-delta);
        const uint64_t d0 = d >> q_num, d1 = d % q_mask;
        for (uint64_t idx = 0; idx < len; ++idx) {
            out[idx] += d0;
            if (idx < d1) out[idx] += 1;
        }
    } else if (delta > 0) {
        uint64_t d = (uint64_t)delta;
        for (uint64_t idx = 0; d != 0; ++idx) {
            if (out[idx & q_mask] == 0) continue;
            out[idx & q_mask] -= 1;
            d -= 1;
        }
    }
    free(p);
    free(n);
    return 0;
}

/* src/register/quant.rs:273-308: idx with no bit above q_mask takes c00 a + c01 b, the others
 * c10 a + c11 b, where a = a[idx & q_mask], b = b[idx & q_mask] (num-complex Mul and Add). */
void oracle_combine_with_unitary(const oc_t* a, const oc_t* b, uint32_t n, const double* c, oc_t* out) {
    const uint64_t q_mask = (1ull << n) - 1;
    const uint64_t len = oracle_reg_len(n + 1);
    const oc_t c00 = {c[0], c[1]}, c01 = {c[2], c[3]}, c10 = {c[4], c[5]}, c11 = {c[6], c[7]};
    for (uint64_t idx = 0; idx < len; ++idx) {
        const oc_t qa = a[q_mask & idx], qb = b[q_mask & idx];
        if ((~q_mask & idx) == 0) out[idx] = c_add(c_mul(c00, qa), c_mul(c01, qb));
        else out[idx] = c_add(c_mul(c10, qa), c_mul(c11, qb));
    }
}

/* src/register/quant.rs:311-328: q.0 = q.0 * c.0 + q.1 * c.1. */
void oracle_linear_composition(oc_t* self, const oc_t* psi, uint64_t len, const double* c) {
    const oc_t c0 = {c[0], c[1]}, c1 = {c[2], c[3]};
    for (uint64_t i = 0; i < len; ++i) self[i] = c_add(c_mul(self[i], c0), c_mul(psi[i], c1));
}

/* ---- builders (src/operator/...) ---------------------------------------------------------- */
/* float-cmp 0.8 `approx_eq!(f64, x, y, ulps = 2)`: equal, within f64::EPSILON, or within 2 ULPs
 * (src/math/approx_cmp.rs:5-10). */
static int approx_eq_real(double x, double y) {
    if (x == y) return 1;
    if (fabs(x - y) <= 2.220446049250313e-16) return 1;
    if ((x < 0) != (y < 0)) return 0;
    int64_t bx, by;
    memcpy(&bx, &x, 8);
    memcpy(&by, &y, 8);
    int64_t d = bx - by;
    if (d < 0) d = -d;
    return d <= 2;
}

static double nsq(oc_t z) { return z.re * z.re + z.im * z.im; }

/* `is_unitary_m1` (src/math/matrix.rs:24-30). */
int oracle_is_unitary_m1(const double* m) {
    oc_t u[4];
    for (int k = 0; k < 4; ++k) { u[k].re = m[2 * k]; u[k].im = m[2 * k + 1]; }
    double e00 = nsq(u[0]) + nsq(u[1]);
    double e11 = nsq(u[2]) + nsq(u[3]);
    oc_t e01 = c_add(c_mul(u[0], c_conj(u[2])), c_mul(u[1], c_conj(u[3])));
    return approx_eq_real(e00, 1.0) && approx_eq_real(e11, 1.0) && approx_eq_real(e01.re + e01.im, 0.0);
}

/* `hermitian_mul` + `is_unitary_m2` (src/math/matrix.rs:37-73). */
static oc_t herm_mul(int i, int j, const oc_t* u) {
    i = (i << 2) & 0xf;
    j = (j << 2) & 0xf;
    if (i == j) {
        oc_t r = {(nsq(u[0 | i]) + nsq(u[1 | i])) + (nsq(u[2 | i]) + nsq(u[3 | i])), 0.0};
        return r;
    }
    return c_add(c_add(c_mul(u[0 | i], c_conj(u[0 | j])), c_mul(u[1 | i], c_conj(u[1 | j]))),
                 c_add(c_mul(u[2 | i], c_conj(u[2 | j])), c_mul(u[3 | i], c_conj(u[3 | j]))));
}

int oracle_is_unitary_m2(const double* m) {
    oc_t u[16];
    for (int k = 0; k < 16; ++k) { u[k].re = m[2 * k]; u[k].im = m[2 * k + 1]; }
    for (int d = 0; d < 4; ++d)
        if (!approx_eq_real(herm_mul(d, d, u).re, 1.0)) return 0;
    for (int a = 0; a < 4; ++a)
        for (int b = a + 1; b < 4; ++b) {
            oc_t e = herm_mul(a, b, u);
            if (!approx_eq_real(e.re + e.im, 0.0)) return 0;
        }
    return 1;
}

static int kind_valid(const qvnt_gate* g) {
    switch (g->kind) {
    case QVNT_GATE_ID: case QVNT_GATE_X: case QVNT_GATE_Y: case QVNT_GATE_Z:
    case QVNT_GATE_S: case QVNT_GATE_T:
        return 1;
    case QVNT_GATE_RX: case QVNT_GATE_RY: case QVNT_GATE_RZ: case QVNT_GATE_H1: case QVNT_GATE_U1:
        return popc(g->a_mask) == 1;
    case QVNT_GATE_RXX: case QVNT_GATE_RYY: case QVNT_GATE_RZZ: case QVNT_GATE_SWAP:
    case QVNT_GATE_ISWAP: case QVNT_GATE_SQRT_SWAP: case QVNT_GATE_SQRT_ISWAP:
        return popc(g->a_mask) == 2;
    case QVNT_GATE_H2: case QVNT_GATE_U2:
        return popc(g->a_mask) == 1 && popc(g->b_mask) == 1 && popc(g->a_mask | g->b_mask) == 2;
    default:
        return 0;
    }
}

int oracle_gate_make(uint32_t kind, uint64_t a_mask, uint64_t b_mask, double angle,
                     const double* matrix, qvnt_gate* out) {
    qvnt_gate g;
    memset(&g, 0, sizeof g);
    g.kind = kind;
    g.a_mask = a_mask;
    if (kind == QVNT_GATE_H2 || kind == QVNT_GATE_U2) g.b_mask = b_mask;
    if (kind == QVNT_GATE_RX || kind == QVNT_GATE_RY || kind == QVNT_GATE_RZ || kind == QVNT_GATE_RXX ||
        kind == QVNT_GATE_RYY || kind == QVNT_GATE_RZZ) {
        double ph = angle;
        ph /= 2.; /* rx.rs:11 `phase /= 2.`; rxx.rs:12 `phase *= 0.5` rounds identically */
        g.phase[0] = cos(ph);
        g.phase[1] = sin(ph);
    }
    if (kind == QVNT_GATE_U1 && matrix) memcpy(g.matrix, matrix, 8 * sizeof(double));
    if (kind == QVNT_GATE_U2 && matrix) memcpy(g.matrix, matrix, 32 * sizeof(double));
    if (!kind_valid(&g)) return QVNT_ERR_BAD_MASK;
    if (kind == QVNT_GATE_U1 && !(matrix && oracle_is_unitary_m1(matrix))) return QVNT_ERR_BAD_ARG;
    if (kind == QVNT_GATE_U2 && !(matrix && oracle_is_unitary_m2(matrix))) return QVNT_ERR_BAD_ARG;
    *out = g;
    return QVNT_OK;
}

void oracle_gate_dgr(qvnt_gate* g) {
    switch (g->kind) {
    case QVNT_GATE_S: case QVNT_GATE_T: case QVNT_GATE_ISWAP: case QVNT_GATE_SQRT_SWAP:
    case QVNT_GATE_SQRT_ISWAP:
        g->dagger = !g->dagger; /* s.rs:39-44 etc. */
        break;
    case QVNT_GATE_RX: case QVNT_GATE_RY: case QVNT_GATE_RZ: case QVNT_GATE_RXX: case QVNT_GATE_RYY:
    case QVNT_GATE_RZZ:
        g->phase[0] = -g->phase[0]; /* rx.rs:42-47: `phase: -self.phase` */
        g->phase[1] = -g->phase[1];
        break;
    case QVNT_GATE_U1: { /* matrix.rs inverse_unitary_m1: conjugate transpose */
        double m[8];
        memcpy(m, g->matrix, sizeof m);
        for (int r = 0; r < 2; ++r)
            for (int c = 0; c < 2; ++c) {
                g->matrix[2 * (2 * r + c)] = m[2 * (2 * c + r)];
                g->matrix[2 * (2 * r + c) + 1] = -m[2 * (2 * c + r) + 1];
            }
        break;
    }
    case QVNT_GATE_U2: { /* matrix.rs inverse_unitary_m2 */
        double m[32];
        memcpy(m, g->matrix, sizeof m);
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) {
                g->matrix[2 * (4 * r + c)] = m[2 * (4 * c + r)];
                g->matrix[2 * (4 * r + c) + 1] = -m[2 * (4 * c + r) + 1];
            }
        break;
    }
    default:
        break;
    }
}

int oracle_gate_c(qvnt_gate* g, uint64_t c_mask) {
    if (((oracle_acts_on(g) | g->ctrl) & c_mask) != 0) return QVNT_ERR_BAD_MASK;
    g->ctrl |= c_mask;
    return QVNT_OK;
}

static size_t push(qvnt_gate* out, size_t n, const qvnt_gate* g) {
    if (out) out[n] = *g;
    return n + 1;
}

size_t oracle_op_h(uint64_t mask, qvnt_gate* out) {
    qvnt_gate g;
    unsigned count = popc(mask);
    if (count == 0) return 0;
    if (count == 1) {
        oracle_gate_make(QVNT_GATE_H1, mask, 0, 0, NULL, &g);
        return push(out, 0, &g);
    }
    size_t n = 0;
    uint64_t i0 = 1, i1 = 0;
    int is_first = 1;
    while (i0 <= mask && i0 != 0) { /* h.rs:25-36 */
        if (i0 & mask) {
            if (is_first) {
                i1 = i0;
                is_first = 0;
            } else {
                oracle_gate_make(QVNT_GATE_H2, i0, i1, 0, NULL, &g);
                n = push(out, n, &g);
                is_first = 1;
            }
        }
        i0 <<= 1;
    }
    if (!is_first) {
        oracle_gate_make(QVNT_GATE_H1, i1, 0, 0, NULL, &g);
        n = push(out, n, &g);
    }
    return n;
}

size_t oracle_op_qft(uint64_t mask, qvnt_gate* out) {
    unsigned count = popc(mask);
    if (count == 0) return 0;
    if (count == 1) return oracle_op_h(mask, out);
    uint64_t vec[64];
    unsigned m = 0;
    for (int i = 0; i < 64; ++i)
        if ((1ull << i) & mask) vec[m++] = 1ull << i;
    size_t n = 0;
    qvnt_gate g;
    for (unsigned i = 0; i + 1 < count; ++i) { /* qft.rs:17-26 */
        n += oracle_op_h(vec[i], out ? out + n : NULL);
        for (unsigned j = 1; j < count - i; ++j) {
            double angle = M_PI * ldexp(1.0, -(int)j); /* PI * 0.5f64.powi(j) */
            oracle_gate_make(QVNT_GATE_RZ, vec[i + j], 0, angle, NULL, &g);
            oracle_gate_c(&g, vec[i]);
            n = push(out, n, &g);
        }
    }
    n += oracle_op_h(vec[count - 1], out ? out + n : NULL);
    return n;
}

size_t oracle_op_qft_swapped(uint64_t mask, qvnt_gate* out) {
    size_t n = oracle_op_qft(mask, out);
    uint64_t vec[64];
    unsigned m = 0;
    for (uint64_t i = 1; i <= mask && i != 0; i <<= 1)
        if (i & mask) vec[m++] = i;
    qvnt_gate g;
    for (unsigned i = 0; i < (m >> 1); ++i) {
        oracle_gate_make(QVNT_GATE_SWAP, vec[i] | vec[m - i - 1], 0, 0, NULL, &g);
        n = push(out, n, &g);
    }
    return n;
}

size_t oracle_op_u3(double the, double phi, double lam, uint64_t mask, qvnt_gate* out) {
    qvnt_gate g; /* operator/mod.rs:499-501: rz(lam) * ry(the) * rz(phi) */
    size_t n = 0;
    oracle_gate_make(QVNT_GATE_RZ, mask, 0, lam, NULL, &g);
    n = push(out, n, &g);
    oracle_gate_make(QVNT_GATE_RY, mask, 0, the, NULL, &g);
    n = push(out, n, &g);
    oracle_gate_make(QVNT_GATE_RZ, mask, 0, phi, NULL, &g);
    n = push(out, n, &g);
    return n;
}

void oracle_ops_dgr(qvnt_gate* gates, size_t count) {
    for (size_t i = 0; i < count / 2; ++i) {
        qvnt_gate t = gates[i];
        gates[i] = gates[count - 1 - i];
        gates[count - 1 - i] = t;
    }
    for (size_t i = 0; i < count; ++i) oracle_gate_dgr(&gates[i]);
}

void oracle_matrix(const qvnt_gate* gates, size_t count, uint32_t size, oc_t* out) {
    uint64_t dim = 1ull << size;
    oc_t* psi = (oc_t*)calloc((size_t)dim, sizeof(oc_t));
    oc_t* tmp = (oc_t*)calloc((size_t)dim, sizeof(oc_t));
    for (uint64_t c = 0; c < dim; ++c) {
        memset(psi, 0, (size_t)dim * sizeof(oc_t));
        psi[c].re = 1.0;
        oracle_apply(gates, count, psi, tmp, dim, 1);
        for (uint64_t r = 0; r < dim; ++r) out[r * dim + c] = psi[r]; /* transpose, :37-43 */
    }
    free(psi);
    free(tmp);
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
