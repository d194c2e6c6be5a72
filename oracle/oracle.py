"""ctypes binding of the oracle (oracle/dsgl_oracle.cpp) -- TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py as the
checker of the CUDA trainer; the product library never loads it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "build", "liboracle.so")

POLICY_REF, POLICY_WINDOW = 0, 1
STORE_F32, STORE_BF16, STORE_F64 = 0, 1, 2


class Config(ctypes.Structure):
    _fields_ = [("d", ctypes.c_int32), ("window", ctypes.c_int32), ("negative", ctypes.c_int32),
                ("iter", ctypes.c_int32), ("workers", ctypes.c_int32), ("threads", ctypes.c_int32),
                ("table_threads", ctypes.c_int32), ("policy", ctypes.c_int32), ("storage", ctypes.c_int32),
                ("schedule", ctypes.c_int32), ("table_size", ctypes.c_int64), ("sample", ctypes.c_float),
                ("alpha", ctypes.c_float), ("sr_seed", ctypes.c_uint64), ("windows", ctypes.c_int32),
                ("pad_", ctypes.c_int32)]


class Stats(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_uint64), ("pairs", ctypes.c_uint64), ("word_count_actual", ctypes.c_uint64),
                ("final_alpha", ctypes.c_float), ("pad_", ctypes.c_float), ("train_seconds", ctypes.c_double)]


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        vp, i32, i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
        L.oracle_train.argtypes = [ctypes.POINTER(Config), vp, i64, vp, i64, vp, vp, ctypes.POINTER(Stats)]
        L.oracle_build_vocab.argtypes = [vp, i64, vp, vp, vp, ctypes.POINTER(ctypes.c_uint64)]
        L.oracle_build_vocab.restype = None
        L.oracle_build_unigram_table.argtypes = [vp, i64, i64, i32, vp]
        L.oracle_build_unigram_table.restype = None
        L.oracle_build_exp_table.argtypes = [vp]
        L.oracle_build_exp_table.restype = None
        L.oracle_init_wih.argtypes = [i64, i32, vp]
        L.oracle_init_wih.restype = None
        L.oracle_lcg_next.argtypes = [ctypes.c_uint64]
        L.oracle_lcg_next.restype = ctypes.c_uint64
        L.oracle_minibatch.argtypes = [i32, i32, i32, i32, i32, vp, ctypes.c_float, vp, vp, vp, vp]
        L.oracle_parse_walks.argtypes = [vp, i64, vp, i64, ctypes.POINTER(i64), ctypes.POINTER(i64),
                                         ctypes.POINTER(i64)]
        L.oracle_parse_walks.restype = i32
        L.oracle_link_scores.argtypes = [i32, i32, vp, i64, vp, i64, vp]
        L.oracle_link_scores.restype = i32
        L.oracle_xlog2x_table.argtypes = [i32, vp]
        L.oracle_xlog2x_table.restype = None
        L.oracle_tanh_pos.argtypes = [ctypes.c_double]
        L.oracle_tanh_pos.restype = ctypes.c_double
        L.oracle_edge_common_neighbors.argtypes = [vp, vp, i64, vp]
        L.oracle_edge_common_neighbors.restype = None
        L.oracle_info_walks.argtypes = [vp, vp, vp, i64, i64, i32, i32, ctypes.c_double, ctypes.c_uint64, i32, vp,
                                        i64, ctypes.POINTER(i64), vp]
        L.oracle_info_walks.restype = i32
        _lib = L
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def f32_to_bf16_rne(x):
    """Round-to-nearest-even fp32 -> bf16 bits (uint16), as the library stores initial rows."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r


def bf16_to_f32(b):
    return (np.asarray(b, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


def vocab(counts):
    counts = np.ascontiguousarray(counts, dtype=np.int32)
    V = len(counts)
    order = np.zeros(V, np.uint32)
    row_of = np.zeros(V, np.int32)
    cns = np.zeros(V, np.int32)
    tw = ctypes.c_uint64()
    lib().oracle_build_vocab(_p(counts), V, _p(order), _p(row_of), _p(cns), ctypes.byref(tw))
    return order, row_of, cns, tw.value


def unigram_table(cn_sorted, table_size, threads):
    cn_sorted = np.ascontiguousarray(cn_sorted, dtype=np.int32)
    t = np.zeros(table_size, np.int32)
    lib().oracle_build_unigram_table(_p(cn_sorted), len(cn_sorted), table_size, threads, _p(t))
    return t


def parse_walks(text):
    """Walk text (bytes) -> (code, tokens int32, max_id, err_pos); code 0 ok, 1 bad byte,
    2 id too long or too large."""
    b = np.frombuffer(bytes(text), dtype=np.uint8)
    n_out, mx, err = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    code = lib().oracle_parse_walks(_p(b) if len(b) else None, len(b), None, 0, ctypes.byref(n_out),
                                    ctypes.byref(mx), ctypes.byref(err))
    out = np.zeros(max(n_out.value, 1), np.int32)
    code = lib().oracle_parse_walks(_p(b) if len(b) else None, len(b), _p(out), len(out), ctypes.byref(n_out),
                                    ctypes.byref(mx), ctypes.byref(err))
    return code, out[:n_out.value], mx.value, err.value


def link_scores(table, pairs):
    """table: [V, d] float32, or uint16 bf16 bits; pairs: [n, 2] int32 rows.
    Returns (scores float32 [n], any pair out of range)."""
    table = np.ascontiguousarray(table)
    pairs = np.ascontiguousarray(pairs, dtype=np.int32)
    dtype = 1 if table.dtype == np.uint16 else 0
    if dtype == 0:
        table = table.astype(np.float32, copy=False)
    V, d = table.shape
    scores = np.zeros(len(pairs), np.float32)
    bad = lib().oracle_link_scores(dtype, d, _p(table), V, _p(pairs) if len(pairs) else None, len(pairs),
                                   _p(scores) if len(pairs) else None)
    return scores, bool(bad)


def exp_table():
    t = np.zeros(1001, np.float32)
    lib().oracle_build_exp_table(_p(t))
    return t


def init_wih(V, d):
    w = np.zeros(V * d, np.float32)
    lib().oracle_init_wih(V, d, _p(w))
    return w.reshape(V, d)


def train(corpus, counts, d=16, window=5, negative=5, iter=1, workers=1, threads=1, table_threads=12,
          policy=POLICY_REF, storage=STORE_F32, table_size=100000000, sample=1e-3, alpha=0.025,
          sr_seed=0x5EED, schedule=0, windows=2):
    """Runs the restated trainer; returns (Wih, Woh, stats) in sorted-row order.

    Wih starts from the reference initialisation (bf16: rounded to nearest even),
    Woh from zeros.  workers > 1 with threads == 1 runs the workers one after another.
    schedule=1 keeps every worker in flight at once (each thread steps its workers
    round-robin), as a GPU runs them: a model of concurrency, not a parity mode.
    """
    corpus = np.ascontiguousarray(corpus, dtype=np.int32)
    counts = np.ascontiguousarray(counts, dtype=np.int32)
    V = len(counts)
    w0 = init_wih(V, d)
    if storage == STORE_F32:
        wih, woh = w0.copy(), np.zeros((V, d), np.float32)
    elif storage == STORE_BF16:
        wih, woh = f32_to_bf16_rne(w0).reshape(V, d), np.zeros((V, d), np.uint16)
    else:
        wih, woh = w0.astype(np.float64), np.zeros((V, d), np.float64)
    cfg = Config(d=d, window=window, negative=negative, iter=iter, workers=workers, threads=threads,
                 table_threads=table_threads, policy=policy, storage=storage, table_size=table_size,
                 sample=sample, alpha=alpha, sr_seed=sr_seed, schedule=schedule, windows=windows)
    st = Stats()
    rc = lib().oracle_train(ctypes.byref(cfg), _p(counts), V, _p(corpus), len(corpus), _p(wih), _p(woh),
                            ctypes.byref(st))
    if rc != 0:
        raise RuntimeError("oracle_train rejected its configuration")
    return wih, woh, {"steps": st.steps, "pairs": st.pairs, "word_count_actual": st.word_count_actual,
                      "final_alpha": st.final_alpha, "train_seconds": st.train_seconds}


def minibatch(inputM, outputM, meta, first, alpha, acc64=False):
    """Reference step on explicit rows: returns (dIn, dOut) as float64 arrays."""
    inputM = np.ascontiguousarray(inputM, dtype=np.float64)
    outputM = np.ascontiguousarray(outputM, dtype=np.float64)
    meta = np.ascontiguousarray(meta, dtype=np.int32)
    I, d = inputM.shape
    O = outputM.shape[0]
    dIn = np.zeros((I, d), np.float64)
    dOut = np.zeros((O, d), np.float64)
    lib().oracle_minibatch(1 if acc64 else 0, d, I, first, O, _p(meta), alpha, _p(inputM), _p(outputM),
                           _p(dIn), _p(dOut))
    return dIn, dOut


def edge_common_neighbors(indptr, indices):
    """cn[e] = |N(u) & N(v)| for every CSR edge e = (u, v) (walk_oracle.cpp)."""
    indptr = np.ascontiguousarray(indptr, dtype=np.int64)
    indices = np.ascontiguousarray(indices, dtype=np.int32)
    cn = np.zeros(len(indices), np.int32)
    lib().oracle_edge_common_neighbors(_p(indptr), _p(indices) if len(indices) else None, len(indptr) - 1,
                                       _p(cn) if len(indices) else None)
    return cn


def info_walks(indptr, indices, cn, walker_num, min_length=20, max_length=80, r_threshold=0.999, seed=1, trace=1):
    """Information-oriented walks restated (walk_oracle.cpp).  Returns (corpus int32 with
    -1 after each walk, lengths int32 per walker)."""
    indptr = np.ascontiguousarray(indptr, dtype=np.int64)
    indices = np.ascontiguousarray(indices, dtype=np.int32)
    cn = np.ascontiguousarray(cn, dtype=np.int32)
    V = len(indptr) - 1
    n = ctypes.c_int64()
    lengths = np.zeros(max(walker_num, 1), np.int32)
    ie = _p(indices) if len(indices) else None
    ce = _p(cn) if len(cn) else None
    lib().oracle_info_walks(_p(indptr), ie, ce, V, walker_num, min_length, max_length, r_threshold, seed, trace, None, 0,
                            ctypes.byref(n), _p(lengths))
    out = np.zeros(max(n.value, 1), np.int32)
    rc = lib().oracle_info_walks(_p(indptr), ie, ce, V, walker_num, min_length, max_length, r_threshold, seed, trace,
                                 _p(out), len(out), ctypes.byref(n), None)
    assert rc == 0
    return out[:n.value], lengths[:walker_num]


def xlog2x_table(n):
    t = np.zeros(n, np.float64)
    lib().oracle_xlog2x_table(n, _p(t))
    return t


def tanh_pos(x):
    return lib().oracle_tanh_pos(float(x))
