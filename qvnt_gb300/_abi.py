"""ctypes binding of the engine's C ABI (include/qvnt_gb300.h).

The library is built in-tree into qvnt_gb300/_build/libqvnt_gb300.so (see qvnt_gb300/build.py).
Loading fails loudly when it is missing: there is no CPU implementation behind this API.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libqvnt_gb300.so")

# enum qvnt_status
OK, ERR_OOM, ERR_BAD_MASK, ERR_BAD_HANDLE, ERR_CUDA, ERR_TIMEOUT, ERR_BAD_ARG, ERR_UNSUPPORTED, ERR_BUSY = range(9)

# enum qvnt_gate_kind (order of qvnt's AtomicOpDispatch, src/operator/atomic/dispatch.rs:82-105)
KINDS = ["ID", "X", "RX", "RXX", "Y", "RY", "RYY", "Z", "S", "T", "RZ", "RZZ", "U1", "U2", "H1", "H2",
         "SWAP", "ISWAP", "SQRT_SWAP", "SQRT_ISWAP"]
KIND = {name: i for i, name in enumerate(KINDS)}

ENGINE_FUSED = 0
ENGINE_PLAIN = 1
ENGINE_PRECISION = 2
ENGINE_TENSOR64 = 3


class QvntGate(ctypes.Structure):
    """`qvnt_gate`: one lowered SingleOp."""

    _fields_ = [
        ("kind", ctypes.c_uint32),
        ("dagger", ctypes.c_uint32),
        ("a_mask", ctypes.c_uint64),
        ("b_mask", ctypes.c_uint64),
        ("ctrl", ctypes.c_uint64),
        ("phase", ctypes.c_double * 2),
        ("matrix", ctypes.c_double * 32),
    ]


assert ctypes.sizeof(QvntGate) == 304

CALL_APPLY, CALL_MEASURE = 0, 1
SUBMIT_KEEP_AMPLITUDES, SUBMIT_DETACHED = 1, 2


class QvntCall(ctypes.Structure):
    """`qvnt_call`: one call of a served request (apply the next gate_count gates, or measure)."""

    _fields_ = [
        ("op", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
        ("gate_count", ctypes.c_uint64),
        ("mask", ctypes.c_uint64),
        ("u01", ctypes.c_double),
    ]


SEP_NOP, SEP_MEASURE, SEP_IF, SEP_RESET = 0, 1, 2, 3
MEASURE_SET, MEASURE_XOR = 0, 1


class QvntBlock(ctypes.Structure):
    """`qvnt_block`: one `(MultiOp, Sep)` block of a runner program."""

    _fields_ = [
        ("sep", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
        ("gate_count", ctypes.c_uint64),
        ("a", ctypes.c_uint64),
        ("b", ctypes.c_uint64),
    ]


class ServerCounters(ctypes.Structure):
    _fields_ = [(name, ctypes.c_uint64) for name in ("submitted", "shed", "completed", "failed", "queued",
                                                      "running", "peak_running", "bytes_active", "bytes_pooled")] + [
        ("now_s", ctypes.c_double)]


class QvntError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s (status %d)" % (message, status))
        self.status = status


class MaskError(QvntError, ValueError):
    """A mask was rejected: qvnt panics or returns None for these."""


_lib = None

P = ctypes.POINTER
c_u32, c_u64, c_int, c_double, c_size = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int, ctypes.c_double, ctypes.c_size_t
c_void = ctypes.c_void_p

_PROTOS = {
    "qvnt_status_string": (ctypes.c_char_p, [c_int]),
    "qvnt_last_error": (ctypes.c_char_p, []),
    "qvnt_abi_version": (c_u32, []),
    "qvnt_ctx_create": (c_int, [c_int, P(c_void)]),
    "qvnt_ctx_destroy": (c_int, [c_void]),
    "qvnt_ctx_mem_info": (c_int, [c_void, P(c_u64), P(c_u64)]),
    "qvnt_reg_create": (c_int, [c_void, c_u32, c_u64, P(c_void)]),
    "qvnt_reg_create_ex": (c_int, [c_void, c_u32, c_u64, c_int, P(c_void)]),
    "qvnt_reg_overlap": (c_int, [c_void, c_void, P(c_double), P(c_double)]),
    "qvnt_reg_sample_all": (c_int, [c_void, c_u64, c_u64, c_void, c_void]),
    "qvnt_reg_combine_with_unitary": (c_int, [c_void, c_void, P(c_double), P(c_void)]),
    "qvnt_reg_linear_composition": (c_int, [c_void, c_void, P(c_double)]),
    "qvnt_precision_plan_info": (c_int, [P(QvntGate), c_size, c_u32, P(c_u64), P(c_u64)]),
    "qvnt_dense_plan_blocks": (c_int, [P(QvntGate), c_size, c_u32, P(c_u64), P(c_double), c_size, P(c_size)]),
    "qvnt_tensor64_mma_costs": (c_int, [c_void, P(c_double), P(c_double), P(c_double)]),
    "qvnt_tensor64_plan_info": (c_int, [P(QvntGate), c_size, c_u32, P(c_u64), P(c_u64)]),
    "qvnt_ctx_set_engine": (c_int, [c_void, c_int]),
    "qvnt_reg_destroy": (c_int, [c_void]),
    "qvnt_reg_clone": (c_int, [c_void, P(c_void)]),
    "qvnt_reg_num": (c_int, [c_void, P(c_u32)]),
    "qvnt_reg_len": (c_int, [c_void, P(c_u64)]),
    "qvnt_reg_set_engine": (c_int, [c_void, c_int]),
    "qvnt_reg_set_fusion_width": (c_int, [c_void, c_u32]),
    "qvnt_reg_apply": (c_int, [c_void, P(QvntGate), c_size]),
    "qvnt_reg_measure_mask": (c_int, [c_void, c_u64, c_double, P(c_u64)]),
    "qvnt_reg_measure_mask_ex": (c_int, [c_void, c_u64, c_double, c_int, P(c_u64)]),
    "qvnt_reg_get_probabilities": (c_int, [c_void, c_void]),
    "qvnt_reg_get_absolute": (c_int, [c_void, P(c_double)]),
    "qvnt_reg_get_polar": (c_int, [c_void, c_void]),
    "qvnt_reg_get_amplitudes": (c_int, [c_void, c_void]),
    "qvnt_reg_get_amplitudes_range": (c_int, [c_void, c_u64, c_u64, c_void]),
    "qvnt_reg_set_amplitudes": (c_int, [c_void, c_void]),
    "qvnt_reg_reset": (c_int, [c_void, c_u64]),
    "qvnt_reg_reset_by_mask": (c_int, [c_void, c_u64]),
    "qvnt_reg_normalize": (c_int, [c_void]),
    "qvnt_reg_tensor": (c_int, [c_void, c_void, P(c_void)]),
    "qvnt_reg_sync": (c_int, [c_void]),
    "qvnt_reg_get_stream": (c_int, [c_void, P(c_void)]),
    "qvnt_apply_host": (c_int, [c_void, P(QvntGate), c_size, c_void, c_void, c_u64]),
    "qvnt_gate_make": (c_int, [c_u32, c_u64, c_u64, c_double, P(c_double), P(QvntGate)]),
    "qvnt_gate_dgr": (c_int, [P(QvntGate)]),
    "qvnt_gate_c": (c_int, [P(QvntGate), c_u64]),
    "qvnt_gate_act_on": (c_u64, [P(QvntGate)]),
    "qvnt_gate_name": (c_int, [P(QvntGate), ctypes.c_char_p, c_size, P(c_size)]),
    "qvnt_op_h": (c_int, [c_u64, P(QvntGate), c_size, P(c_size)]),
    "qvnt_op_qft": (c_int, [c_u64, P(QvntGate), c_size, P(c_size)]),
    "qvnt_op_qft_swapped": (c_int, [c_u64, P(QvntGate), c_size, P(c_size)]),
    "qvnt_op_u2": (c_int, [c_double, c_double, c_u64, P(QvntGate), c_size, P(c_size)]),
    "qvnt_op_u3": (c_int, [c_double, c_double, c_double, c_u64, P(QvntGate), c_size, P(c_size)]),
    "qvnt_ops_dgr": (c_int, [P(QvntGate), c_size]),
    "qvnt_ops_c": (c_int, [P(QvntGate), c_size, c_u64]),
    "qvnt_ops_name": (c_int, [P(QvntGate), c_size, ctypes.c_char_p, c_size, P(c_size)]),
    "qvnt_ops_parse": (c_int, [ctypes.c_char_p, c_size, P(QvntGate), c_size, P(c_size)]),
    "qvnt_wire_encode_gates": (c_int, [P(QvntGate), c_size, c_void, c_size, P(c_size)]),
    "qvnt_wire_decode_gates": (c_int, [c_void, c_size, P(QvntGate), c_size, P(c_size)]),
    "qvnt_plan_info": (c_int, [P(QvntGate), c_size, c_u32, c_u32, P(c_u64), P(c_u64), P(c_u64)]),
    "qvnt_norm_sqr_noalloc": (c_int, [c_void, c_u64, c_void, c_void]),
    "qvnt_reg_stats": (c_int, [c_void, P(c_u64), P(c_u64)]),
    "qvnt_reg_kernel_timing": (c_int, [c_void, c_int, P(c_double), P(c_u64)]),
    "qvnt_workload_random_layers": (c_int, [c_u32, c_u32, P(c_u64), P(QvntGate), c_size, P(c_size)]),
    "qvnt_batch_create": (c_int, [c_void, c_u32, P(c_u32), P(c_u64), P(QvntGate), P(c_u64), P(c_u64), P(c_void)]),
    "qvnt_batch_destroy": (c_int, [c_void]),
    "qvnt_batch_run": (c_int, [c_void, P(c_double), P(c_u64)]),
    "qvnt_batch_set_fusion": (c_int, [c_void, c_u32, c_u32]),
    "qvnt_batch_autotune": (c_int, [c_void, c_u32, P(c_u32), P(c_u32), P(c_double)]),
    "qvnt_batch_get_amplitudes": (c_int, [c_void, c_u32, c_void]),
    "qvnt_batch_info": (c_int, [c_void, P(c_u64), P(c_u64), P(c_u64), P(c_u32), P(c_u32), P(c_double)]),
    "qvnt_server_create": (c_int, [c_void, c_u64, c_u32, c_u32, P(c_void)]),
    "qvnt_server_destroy": (c_int, [c_void]),
    "qvnt_server_clock": (c_int, [c_void, P(c_double)]),
    "qvnt_server_submit": (c_int, [c_void, c_u32, c_u64, P(QvntGate), P(QvntCall), c_u32, c_double, c_int, P(c_u64)]),
    "qvnt_server_wait": (c_int, [c_void, c_u64, c_double, P(c_u64), c_void, P(c_double)]),
    "qvnt_server_stats": (c_int, [c_void, P(ServerCounters)]),
    "qvnt_server_latencies": (c_int, [c_void, P(c_double), c_size, P(c_size)]),
    "qvnt_server_queued_ages": (c_int, [c_void, P(c_double), c_size, P(c_size)]),
    "qvnt_program_run": (c_int, [c_void, c_u32, c_int, P(QvntGate), P(QvntBlock), c_u32, c_u64, P(c_double), c_u32,
                                 P(c_u64), P(c_u32)]),
    "qvnt_qasm_compile": (c_int, [ctypes.c_char_p, c_size, P(c_u32), P(c_u32), P(QvntGate), c_size, P(c_size),
                                  P(QvntBlock), c_u32, P(c_u32), P(c_u64)]),
    "qvnt_program_format": (c_int, [P(QvntGate), P(QvntBlock), c_u32, c_u64, ctypes.c_char_p, c_size, P(c_size)]),
    "qvnt_program_parse": (c_int, [ctypes.c_char_p, c_size, P(QvntGate), c_size, P(c_size), P(QvntBlock), c_u32,
                                   P(c_u32), P(c_u64)]),
    "qvnt_wire_encode_request": (c_int, [c_u32, c_u64, c_int, P(QvntGate), c_size, P(QvntCall), c_u32, c_void,
                                         c_size, P(c_size)]),
    "qvnt_wire_decode_request": (c_int, [c_void, c_size, P(c_u32), P(c_u64), P(c_int), P(QvntGate), c_size,
                                         P(c_size), P(QvntCall), c_u32, P(c_u32)]),
}


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libqvnt_gb300.so is not built (%s); run qvnt_gb300/build.py" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _PROTOS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return list(_PROTOS)


def check(status):
    if status != OK:
        msg = lib().qvnt_last_error().decode(errors="replace")
        if status == ERR_BAD_MASK:
            raise MaskError(status, msg)
        raise QvntError(status, msg)
    return status


def gate_array(gates):
    """A ctypes array of QvntGate from a sequence of QvntGate."""
    arr = (QvntGate * max(len(gates), 1))()
    for i, g in enumerate(gates):
        arr[i] = g
    return arr
