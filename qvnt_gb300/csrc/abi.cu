// C ABI of the engine: contexts, registers, gate validation and dispatch.
//
// Reference boundary: `QReg` (src/register/quant.rs:102-505) and `Applicable::apply`
// (src/operator/applicable.rs:5-15).  The state vector of a register is one device allocation of
// max(2^n, 8) Complex<f64> amplitudes (16 B each, interleaved), owned by the library.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "engine.h"
#include "kernels.h"

namespace qvnt {

namespace {
thread_local std::string g_last_error;
}

int set_error(int status, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

int set_cuda_error(cudaError_t e, const char* what) {
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return set_error(QVNT_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
    }
    return set_error(QVNT_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

static inline unsigned popc(uint64_t x) { return (unsigned)__builtin_popcountll(x); }

uint64_t gate_acts_on(const qvnt_gate& g) {
    switch (g.kind) {
    case QVNT_GATE_ID: return 0;                    // id.rs:15-17
    case QVNT_GATE_H2: return g.a_mask | g.b_mask;  // h2.rs:50-52
    case QVNT_GATE_U2: return g.a_mask;             // u2.rs:70-72 (b_mask omitted)
    default: return g.a_mask;
    }
}

int gate_check_masks(const qvnt_gate& g) {
    switch (g.kind) {
    case QVNT_GATE_ID: case QVNT_GATE_X: case QVNT_GATE_Y: case QVNT_GATE_Z: case QVNT_GATE_S: case QVNT_GATE_T:
        return QVNT_OK;
    case QVNT_GATE_RX: case QVNT_GATE_RY: case QVNT_GATE_RZ: case QVNT_GATE_H1: case QVNT_GATE_U1:
        return popc(g.a_mask) == 1 ? QVNT_OK
                                   : set_error(QVNT_ERR_BAD_MASK, "mask %llu should contain 1 bit",
                                               (unsigned long long)g.a_mask);
    case QVNT_GATE_RXX: case QVNT_GATE_RYY: case QVNT_GATE_RZZ: case QVNT_GATE_SWAP: case QVNT_GATE_ISWAP:
    case QVNT_GATE_SQRT_SWAP: case QVNT_GATE_SQRT_ISWAP:
        return popc(g.a_mask) == 2 ? QVNT_OK
                                   : set_error(QVNT_ERR_BAD_MASK, "mask %llu should contain 2 bits",
                                               (unsigned long long)g.a_mask);
    case QVNT_GATE_H2: case QVNT_GATE_U2:
        return (popc(g.a_mask) == 1 && popc(g.b_mask) == 1 && popc(g.a_mask | g.b_mask) == 2)
                   ? QVNT_OK
                   : set_error(QVNT_ERR_BAD_MASK, "masks %llu, %llu should be two distinct single bits",
                               (unsigned long long)g.a_mask, (unsigned long long)g.b_mask);
    default:
        return set_error(QVNT_ERR_BAD_ARG, "unknown gate kind %u", g.kind);
    }
}

int validate_gate(const qvnt_gate& g, uint64_t len) {
    int st = gate_check_masks(g);
    if (st) return st;
    const uint64_t lim = len - 1;  // qvnt indexes psi[idx ^ mask]: any bit >= log2(len) is out of bounds
    const uint64_t used = g.a_mask | g.b_mask | g.ctrl;
    if (used & ~lim)
        return set_error(QVNT_ERR_BAD_MASK, "gate masks 0x%llx exceed the register (%llu amplitudes)",
                         (unsigned long long)used, (unsigned long long)len);
    if (gate_acts_on(g) & g.ctrl)
        return set_error(QVNT_ERR_BAD_MASK, "control mask 0x%llx overlaps the acting mask 0x%llx",
                         (unsigned long long)g.ctrl, (unsigned long long)gate_acts_on(g));
    return QVNT_OK;
}

DevGate decode_gate(const qvnt_gate& g) {
    DevGate d;
    memset(&d, 0, sizeof d);
    d.kind = g.kind;
    d.dagger = g.dagger ? 1u : 0u;
    d.a = g.a_mask;
    d.b = (g.kind == QVNT_GATE_H2 || g.kind == QVNT_GATE_U2) ? g.b_mask : 0;
    d.ctrl = g.ctrl;
    d.y_ipow = (uint64_t)(uint32_t)(~(uint32_t)(popc(g.a_mask) + 1u));  // y.rs:11
    d.ph_re = g.phase[0];
    d.ph_im = g.phase[1];
    memcpy(d.m, g.matrix, sizeof d.m);
    return d;
}

// ---- register memory ----------------------------------------------------------------------
int reg_alloc(qvnt_reg* r) {
    QVNT_CUDA_TRY(cudaSetDevice(r->ctx->device));
    QVNT_CUDA_TRY(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking));
    cudaError_t e = cudaMalloc(&r->psi, r->len * fmt_bytes(r->fmt));
    if (e != cudaSuccess) {
        r->psi = nullptr;
        return set_cuda_error(e, "cudaMalloc(state)");
    }
    const uint64_t nsc = 2 * chunk_count(r->len) + 8;
    e = cudaMalloc(&r->scratch, nsc * sizeof(double));
    if (e != cudaSuccess) {
        r->scratch = nullptr;
        return set_cuda_error(e, "cudaMalloc(scratch)");
    }
    QVNT_CUDA_TRY(cudaMalloc(&r->d_small, 128));
    QVNT_CUDA_TRY(cudaMemsetAsync(r->d_small, 0, 128, r->stream));
    QVNT_CUDA_TRY(cudaMallocHost(&r->h_small, 64));
    return QVNT_OK;
}

void reg_free(qvnt_reg* r) {
    if (!r) return;
    cudaSetDevice(r->ctx->device);
    if (r->stream) cudaStreamSynchronize(r->stream);
    r->bufs.release();
    if (r->psi) cudaFree(r->psi);
    if (r->alt) cudaFree(r->alt);
    if (r->scratch) cudaFree(r->scratch);
    if (r->staging) cudaFree(r->staging);
    if (r->d_small) cudaFree(r->d_small);
    if (r->h_small) cudaFreeHost(r->h_small);
    for (auto& ev : r->events) {
        cudaEventDestroy(ev.first);
        cudaEventDestroy(ev.second);
    }
    if (r->stream) cudaStreamDestroy(r->stream);
    r->magic = 0;
    delete r;
}

int reg_ensure_alt(qvnt_reg* r) {
    if (r->alt) return QVNT_OK;
    cudaError_t e = cudaMalloc(&r->alt, r->len * sizeof(amp_t));
    if (e != cudaSuccess) {
        r->alt = nullptr;
        return set_cuda_error(e, "cudaMalloc(ping-pong buffer)");
    }
    return QVNT_OK;
}

int reg_ensure_staging(qvnt_reg* r, uint64_t bytes) {
    if (r->staging && r->staging_bytes >= bytes) return QVNT_OK;
    if (r->staging) cudaFree(r->staging);
    r->staging = nullptr;
    cudaError_t e = cudaMalloc(&r->staging, bytes);
    if (e != cudaSuccess) return set_cuda_error(e, "cudaMalloc(staging)");
    r->staging_bytes = bytes;
    return QVNT_OK;
}

// Device-side error flag (d_small + 32): set by a fused kernel whose bounded wait ran out.
int reg_check_device_error(qvnt_reg* r) {
    int* d_err = reinterpret_cast<int*>(reinterpret_cast<char*>(r->d_small) + 32);
    int* h_err = reinterpret_cast<int*>(reinterpret_cast<char*>(r->h_small) + 32);
    QVNT_CUDA_TRY(cudaMemcpyAsync(h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, r->stream));
    QVNT_CUDA_TRY(cudaStreamSynchronize(r->stream));
    if (*h_err) {
        *h_err = 0;
        QVNT_CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), r->stream));
        return set_error(QVNT_ERR_TIMEOUT, "a fused pass gave up waiting for its tile copy; the state is invalid");
    }
    return QVNT_OK;
}

int reg_sync(qvnt_reg* r) {
    QVNT_CUDA_TRY(cudaStreamSynchronize(r->stream));
    return reg_check_device_error(r);
}

// Storage format follows the engine: PLAIN keeps IEEE f64, FUSED keeps double-float pairs.
int reg_set_format(qvnt_reg* r, int fmt) {
    if (r->fmt == fmt) return QVNT_OK;
    int st = launch_convert(r->psi, r->len, fmt == FMT_DF64 ? 1 : 0, r->stream);
    if (st) return st;
    r->fmt = fmt;
    r->launches += 1;
    return QVNT_OK;
}

int timing_begin(qvnt_reg* r, cudaEvent_t* stop) {
    if (!r->timing) return QVNT_OK;
    std::pair<cudaEvent_t, cudaEvent_t> ev;
    QVNT_CUDA_TRY(cudaEventCreate(&ev.first));
    QVNT_CUDA_TRY(cudaEventCreate(&ev.second));
    QVNT_CUDA_TRY(cudaEventRecord(ev.first, r->stream));
    r->events.push_back(ev);
    *stop = ev.second;
    return QVNT_OK;
}

int timing_end(qvnt_reg* r, cudaEvent_t stop) {
    if (!r->timing || !stop) return QVNT_OK;
    QVNT_CUDA_TRY(cudaEventRecord(stop, r->stream));
    return QVNT_OK;
}

// Plain engine: one pass per SingleOp.
int apply_plain(qvnt_reg* r, const qvnt_gate* gates, size_t count) {
    for (size_t k = 0; k < count; ++k) {
        DevGate d = decode_gate(gates[k]);
        if (plain_gate_is_identity(d)) continue;
        cudaEvent_t stop = nullptr;
        int st = timing_begin(r, &stop);
        if (st) return st;
        if (plain_gate_needs_gather(d)) {
            st = reg_ensure_alt(r);
            if (st) return st;
            st = launch_gather_gate(r->psi, r->alt, r->fmt, r->len, d, r->stream, r->ctx->geo);
            std::swap(r->psi, r->alt);
        } else {
            st = launch_plain_gate(r->psi, r->fmt, r->len, d, r->stream, r->ctx->geo);
        }
        if (st) return st;
        st = timing_end(r, stop);
        if (st) return st;
        r->launches += 1;
        r->passes += 1;
    }
    return QVNT_OK;
}

}  // namespace qvnt

using namespace qvnt;

namespace {

constexpr uint32_t kMagicCtx = 0x51435458u;
constexpr uint32_t kMagicReg = 0x51524547u;
constexpr uint32_t kMaxQubits = 40;

inline bool ctx_ok(const qvnt_ctx* c) { return c && c->magic == kMagicCtx; }
inline bool reg_ok(const qvnt_reg* r) { return r && r->magic == kMagicReg; }

}  // namespace

bool qvnt::ctx_valid(const qvnt_ctx* c) { return ctx_ok(c); }

int qvnt::reg_set_priority(qvnt_reg* r, int priority) {
    if (!reg_ok(r)) return set_error(QVNT_ERR_BAD_HANDLE, "invalid register handle");
    QVNT_CUDA_TRY(cudaSetDevice(r->ctx->device));
    cudaStream_t s = nullptr;
    QVNT_CUDA_TRY(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, priority));
    cudaError_t e = cudaStreamSynchronize(r->stream);
    if (e == cudaSuccess) e = cudaStreamDestroy(r->stream);
    if (e != cudaSuccess) {
        cudaStreamDestroy(s);
        return set_cuda_error(e, "stream replacement");
    }
    r->stream = s;
    return QVNT_OK;
}

namespace {

#define CHECK_REG(r) \
    if (!reg_ok(r)) return set_error(QVNT_ERR_BAD_HANDLE, "invalid register handle")
#define CHECK_CTX(c) \
    if (!ctx_ok(c)) return set_error(QVNT_ERR_BAD_HANDLE, "invalid context handle")
#define TRY(expr)              \
    do {                       \
        int _s = (expr);       \
        if (_s) return _s;     \
    } while (0)

uint64_t reg_len_for(uint32_t q_num) {
    uint64_t q = 1ull << q_num;
    return q < 8 ? 8 : q;
}

bool engine_valid(int engine) {
    return engine == QVNT_ENGINE_FUSED || engine == QVNT_ENGINE_PLAIN || engine == QVNT_ENGINE_PRECISION ||
           engine == QVNT_ENGINE_TENSOR64;
}

int fmt_of_engine(int engine) {
    return (engine == QVNT_ENGINE_PLAIN || engine == QVNT_ENGINE_TENSOR64) ? FMT_F64
           : engine == QVNT_ENGINE_PRECISION                               ? FMT_C32
                                                                           : FMT_DF64;
}

int make_reg(qvnt_ctx* ctx, uint32_t q_num, int engine, qvnt_reg** out) {
    qvnt_reg* r = new qvnt_reg();
    r->magic = kMagicReg;
    r->ctx = ctx;
    r->q_num = q_num;
    r->len = reg_len_for(q_num);
    r->engine = engine;
    r->fmt = fmt_of_engine(engine);
    int st = reg_alloc(r);
    if (st) {
        std::string msg = qvnt_last_error();
        reg_free(r);
        return set_error(st, "%s", msg.c_str());
    }
    *out = r;
    return QVNT_OK;
}

}  // namespace

extern "C" {

const char* qvnt_status_string(int status) {
    switch (status) {
    case QVNT_OK: return "ok";
    case QVNT_ERR_OOM: return "out of device memory";
    case QVNT_ERR_BAD_MASK: return "invalid mask";
    case QVNT_ERR_BAD_HANDLE: return "invalid handle";
    case QVNT_ERR_CUDA: return "CUDA error";
    case QVNT_ERR_TIMEOUT: return "device wait timed out";
    case QVNT_ERR_BAD_ARG: return "invalid argument";
    case QVNT_ERR_UNSUPPORTED: return "unsupported";
    case QVNT_ERR_BUSY: return "queue full";
    default: return "unknown status";
    }
}

const char* qvnt_last_error(void) { return qvnt::g_last_error.c_str(); }

uint32_t qvnt_abi_version(void) { return (1u << 16) | 0u; }

int qvnt_ctx_create(int device, qvnt_ctx** out) {
    if (!out) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    // Registers run on their own streams; with the default 8 hardware work queues the kernels of many
    // concurrent registers (the serving loop) serialise in FIFO order behind each other.  32 queues,
    // unless the host set a value; effective only if no CUDA context exists yet in this process.
    setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0);
    int ndev = 0;
    QVNT_CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return set_error(QVNT_ERR_BAD_ARG, "device %d not present (%d)", device, ndev);
    QVNT_CUDA_TRY(cudaSetDevice(device));
    cudaDeviceProp prop;
    QVNT_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
    qvnt_ctx* c = new qvnt_ctx();
    c->magic = kMagicCtx;
    c->device = device;
    c->geo.sms = prop.multiProcessorCount;
    c->geo.blocks_per_sm = 8;
    c->smem_optin = (int)prop.sharedMemPerBlockOptin;
    *out = c;
    return QVNT_OK;
}

int qvnt_ctx_destroy(qvnt_ctx* ctx) {
    CHECK_CTX(ctx);
    if (ctx->host_reg) reg_free(ctx->host_reg);
    ctx->magic = 0;
    delete ctx;
    return QVNT_OK;
}

int qvnt_ctx_mem_info(qvnt_ctx* ctx, uint64_t* free_bytes, uint64_t* total_bytes) {
    CHECK_CTX(ctx);
    size_t f = 0, t = 0;
    QVNT_CUDA_TRY(cudaSetDevice(ctx->device));
    QVNT_CUDA_TRY(cudaMemGetInfo(&f, &t));
    if (free_bytes) *free_bytes = f;
    if (total_bytes) *total_bytes = t;
    return QVNT_OK;
}

int qvnt_ctx_set_engine(qvnt_ctx* ctx, int engine) {
    CHECK_CTX(ctx);
    if (!engine_valid(engine)) return set_error(QVNT_ERR_BAD_ARG, "unknown engine %d", engine);
    std::lock_guard<std::mutex> lock(ctx->host_mu);
    ctx->default_engine = engine;
    if (ctx->host_reg) {  // the scratch register follows on the next qvnt_apply_host call
        reg_free(ctx->host_reg);
        ctx->host_reg = nullptr;
    }
    return QVNT_OK;
}

int qvnt_reg_create(qvnt_ctx* ctx, uint32_t q_num, uint64_t state, qvnt_reg** out) {
    CHECK_CTX(ctx);
    return qvnt_reg_create_ex(ctx, q_num, state, ctx->default_engine, out);
}

int qvnt_reg_create_ex(qvnt_ctx* ctx, uint32_t q_num, uint64_t state, int engine, qvnt_reg** out) {
    CHECK_CTX(ctx);
    if (!out) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    if (q_num > kMaxQubits) return set_error(QVNT_ERR_BAD_ARG, "q_num %u > %u", q_num, kMaxQubits);
    if (!engine_valid(engine)) return set_error(QVNT_ERR_BAD_ARG, "unknown engine %d", engine);
    qvnt_reg* r = nullptr;
    TRY(make_reg(ctx, q_num, engine, &r));
    const uint64_t q_mask = (1ull << q_num) - 1;
    int st = launch_reset(r->psi, r->fmt, r->len, state & q_mask, r->stream);  // quant.rs:129-150
    if (st) {
        reg_free(r);
        return st;
    }
    *out = r;
    return QVNT_OK;
}

int qvnt_reg_destroy(qvnt_reg* reg) {
    CHECK_REG(reg);
    reg_free(reg);
    return QVNT_OK;
}

int qvnt_reg_clone(const qvnt_reg* reg, qvnt_reg** out) {
    CHECK_REG(reg);
    if (!out) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    qvnt_reg* r = nullptr;
    TRY(make_reg(reg->ctx, reg->q_num, reg->engine, &r));
    r->fusion_k = reg->fusion_k;
    cudaError_t e = cudaStreamSynchronize(reg->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(r->psi, reg->psi, r->len * fmt_bytes(r->fmt), cudaMemcpyDeviceToDevice, r->stream);
    if (e != cudaSuccess) {
        reg_free(r);
        return set_cuda_error(e, "clone copy");
    }
    *out = r;
    return QVNT_OK;
}

int qvnt_reg_num(const qvnt_reg* reg, uint32_t* q_num) {
    CHECK_REG(reg);
    if (!q_num) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    *q_num = reg->q_num;
    return QVNT_OK;
}

int qvnt_reg_len(const qvnt_reg* reg, uint64_t* len) {
    CHECK_REG(reg);
    if (!len) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    *len = reg->len;
    return QVNT_OK;
}

int qvnt_reg_set_engine(qvnt_reg* reg, int engine) {
    CHECK_REG(reg);
    if (!engine_valid(engine)) return set_error(QVNT_ERR_BAD_ARG, "unknown engine %d", engine);
    QVNT_CUDA_TRY(cudaSetDevice(reg->ctx->device));
    const int fmt = fmt_of_engine(engine);
    if (fmt_bytes(fmt) != fmt_bytes(reg->fmt)) {
        // element size changes: convert into a new buffer
        double2* nb = nullptr;
        cudaError_t e = cudaMalloc(&nb, reg->len * fmt_bytes(fmt));
        if (e != cudaSuccess) return set_cuda_error(e, "cudaMalloc(state, engine switch)");
        int st = launch_convert_fmt(reg->psi, reg->fmt, nb, fmt, reg->len, reg->stream);
        if (st) {
            cudaFree(nb);
            return st;
        }
        QVNT_CUDA_TRY(cudaStreamSynchronize(reg->stream));
        cudaFree(reg->psi);
        if (reg->alt) cudaFree(reg->alt);
        reg->alt = nullptr;
        reg->psi = nb;
        reg->fmt = fmt;
        reg->launches += 1;
    } else {
        TRY(reg_set_format(reg, fmt));
    }
    reg->engine = engine;
    return QVNT_OK;
}

int qvnt_reg_set_fusion_width(qvnt_reg* reg, uint32_t k) {
    CHECK_REG(reg);
    if (k != 0 && (k < kFusedMinK || k > kFusedMaxK))
        return set_error(QVNT_ERR_BAD_ARG, "fusion width %u outside [%u, %u]", k, kFusedMinK, kFusedMaxK);
    reg->fusion_k = k;
    return QVNT_OK;
}

int qvnt_reg_apply(qvnt_reg* reg, const qvnt_gate* gates, size_t count) {
    CHECK_REG(reg);
    if (count == 0) return QVNT_OK;
    if (!gates) return set_error(QVNT_ERR_BAD_ARG, "null gate list");
    for (size_t k = 0; k < count; ++k) {
        int st = validate_gate(gates[k], reg->len);
        if (st) return set_error(st, "gate %zu: %s", k, qvnt_last_error());
    }
    QVNT_CUDA_TRY(cudaSetDevice(reg->ctx->device));
    if (reg->engine == QVNT_ENGINE_PLAIN) return apply_plain(reg, gates, count);
    if (reg->engine == QVNT_ENGINE_PRECISION) return apply_precision(reg, gates, count);
    if (reg->engine == QVNT_ENGINE_TENSOR64) return apply_tensor64(reg, gates, count);
    return apply_fused(reg, gates, count);
}

int qvnt_reg_measure_mask_ex(qvnt_reg* reg, uint64_t mask, double u01, int renormalise, uint64_t* out_value) {
    CHECK_REG(reg);
    if (!out_value) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    if (!(u01 >= 0.0 && u01 < 1.0)) return set_error(QVNT_ERR_BAD_ARG, "draw %g outside [0, 1)", u01);
    const uint64_t q_mask = (1ull << reg->q_num) - 1;
    mask &= q_mask;  // quant.rs:491
    if (mask == 0) {
        *out_value = 0;
        return QVNT_OK;
    }
    QVNT_CUDA_TRY(cudaSetDevice(reg->ctx->device));
    uint64_t* d_idx = reinterpret_cast<uint64_t*>(reg->d_small);
    int* d_status = reinterpret_cast<int*>(reinterpret_cast<char*>(reg->d_small) + 8);
    QVNT_CUDA_TRY(cudaMemsetAsync(d_status, 0, sizeof(int), reg->stream));
    TRY(launch_measure(reg->psi, reg->fmt, reg->len, q_mask + 1, mask, u01, reg->scratch, d_idx, d_status, renormalise,
                       reg->stream));
    reg->launches += renormalise ? 9 : 6;
    QVNT_CUDA_TRY(cudaMemcpyAsync(reg->h_small, reg->d_small, 16, cudaMemcpyDeviceToHost, reg->stream));
    TRY(reg_sync(reg));
    uint64_t idx;
    int status;
    memcpy(&idx, reg->h_small, 8);
    memcpy(&status, reinterpret_cast<char*>(reg->h_small) + 8, sizeof(int));
    if (status) return set_error(status, "measure_mask: the state has zero or non-finite norm");
    reg->last_measured_index = idx;
    *out_value = idx & mask;  // quant.rs:500
    return QVNT_OK;
}

int qvnt_reg_measure_mask(qvnt_reg* reg, uint64_t mask, double u01, uint64_t* out_value) {
    return qvnt_reg_measure_mask_ex(reg, mask, u01, 0, out_value);
}

int qvnt_reg_get_absolute(qvnt_reg* reg, double* out) {
    CHECK_REG(reg);
    if (!out) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    QVNT_CUDA_TRY(cudaSetDevice(reg->ctx->device));
    double* d_abs = reinterpret_cast<double*>(reg->d_small) + 2;
    TRY(launch_norm_sqr_sum(reg->psi, reg->fmt, reg->len, reg->scratch, d_abs, reg->stream));
    reg->launches += 2;
    QVNT_CUDA_TRY(cudaMemcpyAsync(reg->h_small, d_abs, 8, cudaMemcpyDeviceToHost, reg->stream));
    TRY(reg_sync(reg));
    memcpy(out, reg->h_small, 8);
    return QVNT_OK;
}

int qvnt_reg_get_probabilities(qvnt_reg* reg, double* host_out) {
    CHECK_REG(reg);
    if (!host_out) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    QVNT_CUDA_TRY(cudaSetDevice(reg->ctx->device));
    double* d_abs = reinterpret_cast<double*>(reg->d_small) + 2;
    double* d_inv = d_abs + 1;
    int* d_status = reinterpret_cast<int*>(reinterpret_cast<char*>(reg->d_small) + 8);
    QVNT_CUDA_TRY(cudaMemsetAsync(d_status, 0, sizeof(int), reg->stream));
    TRY(launch_norm_sqr_sum(reg->psi, reg->fmt, reg->len, reg->scratch, d_abs, reg->stream));
    TRY(launch_inv(d_abs, d_inv, d_status, reg->stream));
    const uint64_t q_size = 1ull << reg->q_num;
    const uint64_t piece = q_size < (1ull << 23) ? q_size : (1ull << 23);
    TRY(reg_ensure_staging(reg, piece * sizeof(double)));
    for (uint64_t first = 0; first < q_size; first += piece) {
        const uint64_t n = (q_size - first) < piece ? (q_size - first) : piece;
        TRY(launch_probabilities(reg->psi, reg->fmt, first, n, d_inv, reinterpret_cast<double*>(reg->staging),
                                 reg->stream));
        QVNT_CUDA_TRY(cudaMemcpyAsync(host_out + first, reg->staging, n * sizeof(double), cudaMemcpyDeviceToHost,
                                      reg->stream));
        QVNT_CUDA_TRY(cudaStreamSynchronize(reg->stream));
        reg->launches += 1;
    }
    reg->launches += 3;
    return QVNT_OK;
}

int qvnt_reg_get_polar(qvnt_reg* reg, double* host_out) {
    CHECK_REG(reg);
    if (!host_out) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    QVNT_CUDA_TRY(cudaSetDevice(reg->ctx->device));
    const uint64_t q_size = 1ull << reg->q_num;
    const uint64_t piece = q_size < (1ull << 22) ? q_size : (1ull << 22);
    TRY(reg_ensure_staging(reg, piece * 2 * sizeof(double)));
    for (uint64_t first = 0; first < q_size; first += piece) {
        const uint64_t n = (q_size - first) < piece ? (q_size - first) : piece;
        TRY(launch_polar(reg->psi, reg->fmt, first, n, reinterpret_cast<double*>(reg->staging), reg->stream));
        QVNT_CUDA_TRY(cudaMemcpyAsync(host_out + 2 * first, reg->staging, 2 * n * sizeof(double),
                                      cudaMemcpyDeviceToHost, reg->stream));
        QVNT_CUDA_TRY(cudaStreamSynchronize(reg->stream));
        reg->launches += 1;
    }
    return QVNT_OK;
}

// Device -> host copy of amplitudes [first, first + count) as IEEE f64.  Double-float registers
// are converted piecewise through the staging buffer; the state itself is not modified.
static int copy_amplitudes_out(qvnt_reg* reg, uint64_t first, uint64_t count, double* host_out) {
    if (reg->fmt == FMT_F64) {
        QVNT_CUDA_TRY(cudaMemcpyAsync(host_out, reg->psi + first, count * sizeof(amp_t), cudaMemcpyDeviceToHost,
                                      reg->stream));
        return reg_sync(reg);
    }
    const uint64_t piece = count < (1ull << 22) ? count : (1ull << 22);
    TRY(reg_ensure_staging(reg, piece * sizeof(amp_t)));
    for (uint64_t at = 0; at < count; at += piece) {
        const uint64_t n = (count - at) < piece ? (count - at) : piece;
        TRY(launch_copy_out(reg->psi, reg->fmt, first + at, n, reinterpret_cast<double2*>(reg->staging), reg->stream));
        QVNT_CUDA_TRY(cudaMemcpyAsync(host_out + 2 * at, reg->staging, n * sizeof(amp_t), cudaMemcpyDeviceToHost,
                                      reg->stream));
        TRY(reg_sync(reg));
        reg->launches += 1;
    }
    return QVNT_OK;
}

int qvnt_reg_get_amplitudes(qvnt_reg* reg, double* host_out) {
    CHECK_REG(reg);
    if (!host_out) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    QVNT_CUDA_TRY(cudaSetDevice(reg->ctx->device));
    return copy_amplitudes_out(reg, 0, reg->len, host_out);
}

int qvnt_reg_get_amplitudes_range(qvnt_reg* reg, uint64_t first, uint64_t count, double* host_out) {
    CHECK_REG(reg);
    if (!host_out && count) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    if (first > reg->len || count > reg->len - first)
        return set_error(QVNT_ERR_BAD_ARG, "range [%llu, +%llu) outside %llu amplitudes", (unsigned long long)first,
                         (unsigned long long)count, (unsigned long long)reg->len);
    if (count == 0) return QVNT_OK;
    QVNT_CUDA_TRY(cudaSetDevice(reg->ctx->device));
    return copy_amplitudes_out(reg, first, count, host_out);
}

int qvnt_reg_set_amplitudes(qvnt_reg* reg, const double* host_in) {
    CHECK_REG(reg);
    if (!host_in) return set_error(QVNT_ERR_BAD_ARG, "null input pointer");
    QVNT_CUDA_TRY(cudaSetDevice(reg->ctx->device));
    if (reg->fmt == FMT_C32) {  // through the staging buffer, piecewise
        const uint64_t piece = reg->len < (1ull << 22) ? reg->len : (1ull << 22);
        TRY(reg_ensure_staging(reg, piece * sizeof(amp_t)));
        for (uint64_t at = 0; at < reg->len; at += piece) {
            const uint64_t n = (reg->len - at) < piece ? (reg->len - at) : piece;
            QVNT_CUDA_TRY(cudaMemcpyAsync(reg->staging, host_in + 2 * at, n * sizeof(amp_t), cudaMemcpyHostToDevice,
                                          reg->stream));
            TRY(launch_copy_in(reg->psi, reg->fmt, at, n, reinterpret_cast<const double2*>(reg->staging), reg->stream));
            TRY(reg_sync(reg));
            reg->launches += 1;
        }
        return QVNT_OK;
    }
    QVNT_CUDA_TRY(cudaMemcpyAsync(reg->psi, host_in, reg->len * sizeof(amp_t), cudaMemcpyHostToDevice, reg->stream));
    if (reg->fmt == FMT_DF64) {
        TRY(launch_convert(reg->psi, reg->len, 1, reg->stream));  // f64 -> double-float, in place
        reg->launches += 1;
    }
    return reg_sync(reg);
}

int qvnt_reg_reset(qvnt_reg* reg, uint64_t state) {
    CHECK_REG(reg);
    QVNT_CUDA_TRY(cudaSetDevice(reg->ctx->device));
    const uint64_t q_mask = (1ull << reg->q_num) - 1;
    TRY(launch_reset(reg->psi, reg->fmt, reg->len, state & q_mask, reg->stream));  // quant.rs:202-205
    reg->launches += 1;
    return QVNT_OK;
}

int qvnt_reg_normalize(qvnt_reg* reg) {
    CHECK_REG(reg);
    QVNT_CUDA_TRY(cudaSetDevice(reg->ctx->device));
    double* d_abs = reinterpret_cast<double*>(reg->d_small) + 2;
    TRY(launch_norm_sqr_sum(reg->psi, reg->fmt, reg->len, reg->scratch, d_abs, reg->stream));
    TRY(launch_normalize(reg->psi, reg->fmt, reg->len, d_abs, reg->stream));
    reg->launches += 3;
    return QVNT_OK;
}

int qvnt_reg_reset_by_mask(qvnt_reg* reg, uint64_t mask) {
    CHECK_REG(reg);
    const uint64_t q_mask = (1ull << reg->q_num) - 1;
    if ((mask & q_mask) == q_mask) return qvnt_reg_reset(reg, 0);  // quant.rs:208-210
    QVNT_CUDA_TRY(cudaSetDevice(reg->ctx->device));
    TRY(launch_zero_mask(reg->psi, reg->fmt, reg->len, mask, reg->stream));
    reg->launches += 1;
    return qvnt_reg_normalize(reg);
}

int qvnt_reg_tensor(const qvnt_reg* a, const qvnt_reg* b, qvnt_reg** out) {
    CHECK_REG(a);
    CHECK_REG(b);
    if (!out) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    if (a->ctx != b->ctx) return set_error(QVNT_ERR_BAD_ARG, "registers belong to different contexts");
    if (a->fmt == FMT_C32 || b->fmt == FMT_C32)
        return set_error(QVNT_ERR_UNSUPPORTED, "tensor product of precision-engine registers");
    const uint32_t q_num = a->q_num + b->q_num;
    if (q_num > kMaxQubits) return set_error(QVNT_ERR_BAD_ARG, "tensor product has %u qubits", q_num);
    QVNT_CUDA_TRY(cudaSetDevice(a->ctx->device));
    QVNT_CUDA_TRY(cudaStreamSynchronize(a->stream));
    QVNT_CUDA_TRY(cudaStreamSynchronize(b->stream));
    qvnt_reg* r = nullptr;
    TRY(make_reg(a->ctx, q_num, a->engine, &r));
    int st = launch_tensor(a->psi, a->fmt, a->q_num, b->psi, b->fmt, b->q_num, r->psi, r->fmt, r->len, r->stream);
    if (st) {
        reg_free(r);
        return st;
    }
    r->launches += 1;
    *out = r;
    return QVNT_OK;
}

int qvnt_reg_sync(qvnt_reg* reg) {
    CHECK_REG(reg);
    QVNT_CUDA_TRY(cudaSetDevice(reg->ctx->device));
    return reg_sync(reg);
}

int qvnt_apply_host(qvnt_ctx* ctx, const qvnt_gate* gates, size_t count, const double* psi_i, double* psi_o,
                    uint64_t len) {
    CHECK_CTX(ctx);
    if (!psi_i || !psi_o) return set_error(QVNT_ERR_BAD_ARG, "null host buffer");
    if (len < 8 || (len & (len - 1)) != 0) return set_error(QVNT_ERR_BAD_ARG, "len %llu is not a power of two >= 8",
                                                             (unsigned long long)len);
    uint32_t q_num = (uint32_t)__builtin_ctzll(len);
    if (q_num > kMaxQubits) return set_error(QVNT_ERR_BAD_ARG, "len too large");
    std::lock_guard<std::mutex> lock(ctx->host_mu);
    if (ctx->host_reg && ctx->host_reg->len != len) {
        reg_free(ctx->host_reg);
        ctx->host_reg = nullptr;
    }
    if (!ctx->host_reg)
        TRY(make_reg(ctx, q_num, ctx->default_engine == QVNT_ENGINE_PRECISION ? QVNT_ENGINE_FUSED : ctx->default_engine,
                     &ctx->host_reg));
    qvnt_reg* r = ctx->host_reg;
    for (size_t k = 0; k < count; ++k) {
        int st = validate_gate(gates[k], r->len);
        if (st) return set_error(st, "gate %zu: %s", k, qvnt_last_error());
    }
    QVNT_CUDA_TRY(cudaSetDevice(ctx->device));
    // The plugin register is scratch: its storage is converted in place around the gate passes (and
    // left as IEEE f64 afterwards: the next call overwrites it).
    QVNT_CUDA_TRY(cudaMemcpyAsync(r->psi, psi_i, len * sizeof(amp_t), cudaMemcpyHostToDevice, r->stream));
    if (r->fmt == FMT_DF64) TRY(launch_convert(r->psi, r->len, 1, r->stream));
    TRY(r->engine == QVNT_ENGINE_PLAIN      ? apply_plain(r, gates, count)
        : r->engine == QVNT_ENGINE_TENSOR64 ? apply_tensor64(r, gates, count)
                                            : apply_fused(r, gates, count));
    if (r->fmt == FMT_DF64) TRY(launch_convert(r->psi, r->len, 0, r->stream));
    QVNT_CUDA_TRY(cudaMemcpyAsync(psi_o, r->psi, len * sizeof(amp_t), cudaMemcpyDeviceToHost, r->stream));
    r->launches += r->fmt == FMT_DF64 ? 2 : 0;
    return reg_sync(r);
}

int qvnt_reg_get_stream(const qvnt_reg* reg, void** stream) {
    CHECK_REG(reg);
    if (!stream) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    *stream = reinterpret_cast<void*>(reg->stream);
    return QVNT_OK;
}

int qvnt_reg_sample_all(qvnt_reg* reg, uint64_t count, uint64_t seed, const double* normals, uint64_t* out_counts) {
    CHECK_REG(reg);
    if (!out_counts) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    const uint64_t q_size = 1ull << reg->q_num;
    if (reg->len != q_size || q_size < 2)  // quant.rs:515-538 indexes p (2^n entries) over psi.len()
        return set_error(QVNT_ERR_BAD_ARG, "sample_all needs at least 3 qubits (qvnt panics below)");
    QVNT_CUDA_TRY(cudaSetDevice(reg->ctx->device));
    const uint64_t nc = chunk_count(q_size);
    double* d_abs = reg->scratch + 2 * nc;
    double* d_inv = d_abs + 1;
    double* d_nsum = d_abs + 2;
    int* d_status = reinterpret_cast<int*>(reinterpret_cast<char*>(reg->d_small) + 8);
    double* d_n = nullptr;
    double* d_z = nullptr;
    cudaError_t e = cudaMalloc(&d_n, q_size * sizeof(double));
    if (e == cudaSuccess && normals) e = cudaMalloc(&d_z, q_size * sizeof(double));
    if (e == cudaSuccess && normals)
        e = cudaMemcpyAsync(d_z, normals, q_size * sizeof(double), cudaMemcpyHostToDevice, reg->stream);
    int st = QVNT_OK;
    std::vector<long long> h(q_size);
    if (e == cudaSuccess) {
        st = launch_norm_sqr_sum(reg->psi, reg->fmt, reg->len, reg->scratch, d_abs, reg->stream);
        if (!st) st = launch_inv(d_abs, d_inv, d_status, reg->stream);
        if (!st) st = launch_sample_all(reg->psi, reg->fmt, q_size, d_inv, d_z, seed, count, d_n, reg->scratch, d_nsum,
                                        reg->stream);
        if (!st) e = cudaMemcpyAsync(h.data(), d_n, q_size * sizeof(long long), cudaMemcpyDeviceToHost, reg->stream);
        if (!st && e == cudaSuccess) e = cudaStreamSynchronize(reg->stream);
        reg->launches += 6;
    }
    if (d_n) cudaFree(d_n);
    if (d_z) cudaFree(d_z);
    if (st) return st;
    if (e != cudaSuccess) return set_cuda_error(e, "sample_all");
    // correction of the total to `count` (quant.rs:562-591), sequential as there
    const uint64_t q_mask = q_size - 1;
    long long total = 0;
    for (uint64_t i = 0; i < q_size; ++i) {
        out_counts[i] = (uint64_t)h[i];
        total += h[i];
    }
    const long long delta = total - (long long)count;
    if (delta < 0) {
        const uint64_t d = (uint64_t)(-delta);
        const uint64_t d0 = d >> reg->q_num, d1 = d % q_mask;
        for (uint64_t idx = 0; idx < q_size; ++idx) out_counts[idx] += d0 + (idx < d1 ? 1 : 0);
    } else if (delta > 0) {
        uint64_t d = (uint64_t)delta;
        for (uint64_t idx = 0; d != 0; ++idx) {
            if (out_counts[idx & q_mask] == 0) continue;
            out_counts[idx & q_mask] -= 1;
            d -= 1;
        }
    }
    return QVNT_OK;
}

int qvnt_reg_combine_with_unitary(const qvnt_reg* a, const qvnt_reg* b, const double* c, qvnt_reg** out) {
    CHECK_REG(a);
    CHECK_REG(b);
    if (!c || !out) return set_error(QVNT_ERR_BAD_ARG, "null argument");
    if (a->ctx != b->ctx) return set_error(QVNT_ERR_BAD_ARG, "registers belong to different contexts");
    if (a->q_num != b->q_num)  // quant.rs:277: None
        return set_error(QVNT_ERR_BAD_ARG, "registers of %u and %u qubits", a->q_num, b->q_num);
    if (a->fmt == FMT_C32 || b->fmt == FMT_C32)
        return set_error(QVNT_ERR_UNSUPPORTED, "combine of precision-engine registers");
    if (a->q_num + 1 > kMaxQubits) return set_error(QVNT_ERR_BAD_ARG, "result too large");
    qvnt_gate chk;
    TRY(qvnt_gate_make(QVNT_GATE_U1, 1, 0, 0.0, c, &chk));  // quant.rs:275: is_unitary_m1
    QVNT_CUDA_TRY(cudaSetDevice(a->ctx->device));
    QVNT_CUDA_TRY(cudaStreamSynchronize(a->stream));
    QVNT_CUDA_TRY(cudaStreamSynchronize(b->stream));
    qvnt_reg* r = nullptr;
    TRY(make_reg(a->ctx, a->q_num + 1, a->engine, &r));
    int st = launch_combine(a->psi, a->fmt, b->psi, b->fmt, a->q_num, c, r->psi, r->fmt, r->len, r->stream);
    if (st) {
        reg_free(r);
        return st;
    }
    r->launches += 1;
    *out = r;
    return QVNT_OK;
}

int qvnt_reg_linear_composition(qvnt_reg* self, const qvnt_reg* psi, const double* c) {
    CHECK_REG(self);
    CHECK_REG(psi);
    if (!c) return set_error(QVNT_ERR_BAD_ARG, "null coefficients");
    if (self->len != psi->len)  // quant.rs:312: assert_eq!
        return set_error(QVNT_ERR_BAD_ARG, "buffers of %llu and %llu amplitudes", (unsigned long long)self->len,
                         (unsigned long long)psi->len);
    if (self->fmt == FMT_C32 || psi->fmt == FMT_C32)
        return set_error(QVNT_ERR_UNSUPPORTED, "linear composition of precision-engine registers");
    QVNT_CUDA_TRY(cudaSetDevice(self->ctx->device));
    QVNT_CUDA_TRY(cudaStreamSynchronize(psi->stream));
    TRY(launch_linear(self->psi, self->fmt, psi->psi, psi->fmt, self->len, c, self->stream));
    self->launches += 1;
    return QVNT_OK;
}

int qvnt_reg_overlap(const qvnt_reg* a, const qvnt_reg* b, double* fidelity, double* max_abs_diff) {
    CHECK_REG(a);
    CHECK_REG(b);
    if (a->len != b->len) return set_error(QVNT_ERR_BAD_ARG, "registers of different sizes");
    if (a->ctx != b->ctx) return set_error(QVNT_ERR_BAD_ARG, "registers belong to different contexts");
    QVNT_CUDA_TRY(cudaSetDevice(a->ctx->device));
    QVNT_CUDA_TRY(cudaStreamSynchronize(b->stream));
    double* d = nullptr;
    const uint64_t nc = chunk_count(a->len);
    QVNT_CUDA_TRY(cudaMalloc(&d, (5 * nc + 8) * sizeof(double)));
    int st = launch_overlap(a->psi, a->fmt, b->psi, b->fmt, a->len, d + 8, d, a->stream);
    double h[5] = {0, 0, 0, 0, 0};
    cudaError_t e = st ? cudaSuccess : cudaMemcpyAsync(h, d, sizeof h, cudaMemcpyDeviceToHost, a->stream);
    if (e == cudaSuccess && !st) e = cudaStreamSynchronize(a->stream);
    cudaFree(d);
    if (st) return st;
    if (e != cudaSuccess) return set_cuda_error(e, "overlap");
    // |<a|b>|^2 / (<a|a> <b|b>)
    if (fidelity) *fidelity = (h[2] > 0 && h[3] > 0) ? (h[0] * h[0] + h[1] * h[1]) / (h[2] * h[3]) : 0.0;
    if (max_abs_diff) *max_abs_diff = h[4];
    return QVNT_OK;
}

int qvnt_precision_plan_info(const qvnt_gate* gates, size_t count, uint32_t q_num, uint64_t* passes,
                             uint64_t* blocks) {
    if (!gates && count) return set_error(QVNT_ERR_BAD_ARG, "null gate list");
    if (!passes || !blocks) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    if (q_num < 12 || q_num > kMaxQubits) return set_error(QVNT_ERR_BAD_ARG, "q_num %u outside [12, %u]", q_num, kMaxQubits);
    for (size_t k = 0; k < count; ++k) {
        int st = validate_gate(gates[k], 1ull << q_num);
        if (st) return set_error(st, "gate %zu: %s", k, qvnt_last_error());
    }
    return precision_plan_info(gates, count, q_num, passes, blocks);
}

int qvnt_tensor64_plan_info(const qvnt_gate* gates, size_t count, uint32_t q_num, uint64_t* passes,
                            uint64_t* plain_gates) {
    if (!gates && count) return set_error(QVNT_ERR_BAD_ARG, "null gate list");
    if (!passes || !plain_gates) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    if (q_num > kMaxQubits) return set_error(QVNT_ERR_BAD_ARG, "q_num %u > %u", q_num, kMaxQubits);
    const uint64_t len = q_num < 3 ? 8 : 1ull << q_num;
    for (size_t k = 0; k < count; ++k) {
        int st = validate_gate(gates[k], len);
        if (st) return set_error(st, "gate %zu: %s", k, qvnt_last_error());
    }
    return tensor64_plan_info(gates, count, (uint32_t)__builtin_ctzll(len), passes, plain_gates);
}

int qvnt_tensor64_mma_costs(qvnt_ctx* ctx, double* n64_cycles, double* n256_cycles, double* tile_cycles) {
    CHECK_CTX(ctx);
    if (!n64_cycles || !n256_cycles || !tile_cycles) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    return tensor64_mma_costs(ctx->device, ctx->geo.sms, n64_cycles, n256_cycles, tile_cycles);
}

int qvnt_dense_plan_blocks(const qvnt_gate* gates, size_t count, uint32_t q_num, uint64_t* sups, double* mats,
                           size_t cap, size_t* nblocks) {
    if (!gates && count) return set_error(QVNT_ERR_BAD_ARG, "null gate list");
    if (!nblocks) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    if (q_num < 5 || q_num > kMaxQubits) return set_error(QVNT_ERR_BAD_ARG, "q_num %u outside 5..%u", q_num, kMaxQubits);
    if (cap && (!sups || !mats)) return set_error(QVNT_ERR_BAD_ARG, "null block buffers");
    const uint64_t len = 1ull << q_num;
    for (size_t k = 0; k < count; ++k) {
        int st = validate_gate(gates[k], len);
        if (st) return set_error(st, "gate %zu: %s", k, qvnt_last_error());
    }
    return tensor64_plan_blocks(gates, count, q_num, sups, mats, cap, nblocks);
}

int qvnt_reg_stats(const qvnt_reg* reg, uint64_t* kernel_launches, uint64_t* passes) {
    CHECK_REG(reg);
    if (kernel_launches) *kernel_launches = reg->launches;
    if (passes) *passes = reg->passes;
    return QVNT_OK;
}

int qvnt_reg_kernel_timing(qvnt_reg* reg, int enable, double* ms, uint64_t* launches) {
    CHECK_REG(reg);
    QVNT_CUDA_TRY(cudaSetDevice(reg->ctx->device));
    QVNT_CUDA_TRY(cudaStreamSynchronize(reg->stream));
    double total = 0.0;
    for (auto& ev : reg->events) {
        float t = 0.f;
        QVNT_CUDA_TRY(cudaEventElapsedTime(&t, ev.first, ev.second));
        total += t;
    }
    if (ms) *ms = total;
    if (launches) *launches = reg->events.size();
    if (enable >= 0) {
        for (auto& ev : reg->events) {
            cudaEventDestroy(ev.first);
            cudaEventDestroy(ev.second);
        }
        reg->events.clear();
        reg->timing = enable != 0;
    }
    return QVNT_OK;
}

}  // extern "C"
