// Internal structures shared by the C ABI (abi.cu) and the fused engine (fused.cu).
#pragma once

#include <mutex>
#include <utility>
#include <vector>

#include "common.cuh"

namespace qvnt {

// Fused-pass tile widths accepted by qvnt_reg_set_fusion_width.
constexpr uint32_t kFusedMinK = 6;
constexpr uint32_t kFusedMaxK = 13;

// Buffers an engine keeps between apply calls (the dense-block weights of the precision and tensor
// engines: a device buffer and its pinned host mirror for the upload).  They grow to powers of two and
// never synchronise the device while they grow: the device buffer is stream-ordered (allocated and
// freed on the register's stream), and an outgrown pinned buffer is kept until the register is freed
// (freeing pinned memory waits for the whole device, which would stall every other stream of a server).
struct EngineBuffers {
    void* d_buf = nullptr;
    size_t d_bytes = 0;
    void* h_buf = nullptr;  // pinned host mirror for the upload
    size_t h_bytes = 0;
    std::vector<void*> retired;      // outgrown pinned mirrors, freed with the register
    cudaEvent_t uploaded = nullptr;  // recorded on the register's stream after the last upload from h_buf
    void release();
    // Buffers of at least `bytes`; h_buf may be written once this returns (the last upload from it is
    // done: the host waits for that upload only, not for the stream's other work).
    int acquire(size_t bytes, cudaStream_t stream);
    // Queues the upload of `bytes` from h_buf to d_buf on `stream` and records `uploaded`.
    int upload(size_t bytes, cudaStream_t stream);
};

}  // namespace qvnt

struct qvnt_ctx {
    uint32_t magic = 0;
    int device = 0;
    qvnt::Geometry geo;
    int smem_optin = 0;
    int default_engine = QVNT_ENGINE_TENSOR64;  // f64 semantics by default
    std::mutex host_mu;
    struct qvnt_reg* host_reg = nullptr;  // scratch register of qvnt_apply_host
};

struct qvnt_reg {
    uint32_t magic = 0;
    qvnt_ctx* ctx = nullptr;
    uint32_t q_num = 0;
    uint64_t len = 0;  // max(2^q_num, 8) amplitudes
    qvnt::amp_t* psi = nullptr;
    qvnt::amp_t* alt = nullptr;  // lazily allocated second buffer (out-of-place passes)
    double* scratch = nullptr;   // reduction partials
    void* staging = nullptr;     // device staging for host reads
    uint64_t staging_bytes = 0;
    void* d_small = nullptr;     // 128 B: device results (index, status, sums), then the tensor engine's scale ring
    void* h_small = nullptr;     // pinned 64 B host mirror
    cudaStream_t stream = nullptr;
    int engine = QVNT_ENGINE_FUSED;
    int fmt = 0;  // storage format (kernels.h Fmt): follows the engine
    uint32_t fusion_k = 0;
    uint64_t launches = 0;
    uint64_t passes = 0;
    uint64_t last_measured_index = 0;
    bool timing = false;
    bool tile_grid = false;  // one CTA per tile instead of a persistent grid (shared-GPU serving)
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> events;
    qvnt::EngineBuffers bufs;
};

namespace qvnt {
bool ctx_valid(const qvnt_ctx* c);
int reg_set_priority(qvnt_reg* r, int priority);  // replaces the register's stream by one of this priority
int validate_gate(const qvnt_gate& g, uint64_t len);
uint64_t gate_acts_on(const qvnt_gate& g);
int gate_check_masks(const qvnt_gate& g);
DevGate decode_gate(const qvnt_gate& g);
int reg_ensure_alt(qvnt_reg* r);
int reg_sync(qvnt_reg* r);
int timing_begin(qvnt_reg* r, cudaEvent_t* stop);
int timing_end(qvnt_reg* r, cudaEvent_t stop);
int apply_plain(qvnt_reg* r, const qvnt_gate* gates, size_t count);
int apply_fused(qvnt_reg* r, const qvnt_gate* gates, size_t count);
int apply_precision(qvnt_reg* r, const qvnt_gate* gates, size_t count);
int precision_plan_info(const qvnt_gate* gates, size_t count, uint32_t L, uint64_t* passes, uint64_t* blocks);
int apply_tensor64(qvnt_reg* r, const qvnt_gate* gates, size_t count);
int tensor64_plan_info(const qvnt_gate* gates, size_t count, uint32_t L, uint64_t* passes, uint64_t* plain_gates);
int tensor64_mma_costs(int device, int sms, double* n64, double* n256, double* tile);
int tensor64_plan_blocks(const qvnt_gate* gates, size_t count, uint32_t L, uint64_t* sups, double* mats, size_t cap,
                         size_t* nblocks);
int launch_inv(const double* d_abs, double* d_inv, int* d_status, cudaStream_t stream);
}  // namespace qvnt
