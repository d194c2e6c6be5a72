"""ctypes binding of libsgns.so (include/sgns.h) for tests, benchmarks and scripting.

The trainer itself is C++/CUDA behind the C ABI; this module only marshals arguments.
Loading fails loudly when the shared library has not been built: there is no fallback.
"""
import ctypes
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "build", "libsgns.so")
HEADER = os.path.join(ROOT, "include", "sgns.h")

OK, EINVAL, ENOMEM, ECUDA, ETIMEOUT, EIO, ESTATE = range(7)
STORE_FP32, STORE_BF16_SR = 0, 1
ENGINE_PLAIN, ENGINE_PERSISTENT = 0, 1
MODE_HOGWILD, MODE_REPLAY_EXACT = 0, 1


class Options(ctypes.Structure):
    _fields_ = [
        ("size", ctypes.c_int32), ("window", ctypes.c_int32), ("negative", ctypes.c_int32),
        ("batch_size", ctypes.c_int32), ("sample", ctypes.c_float), ("alpha", ctypes.c_float),
        ("min_count", ctypes.c_int32), ("iter", ctypes.c_int32), ("threads", ctypes.c_int32),
        ("debug", ctypes.c_int32), ("binary", ctypes.c_int32), ("storage", ctypes.c_int32),
        ("engine", ctypes.c_int32), ("workers", ctypes.c_int32), ("warps_per_cta", ctypes.c_int32),
        ("device", ctypes.c_int32), ("compute_loss", ctypes.c_int32), ("mode", ctypes.c_int32),
        ("table_size", ctypes.c_int64), ("seed", ctypes.c_uint64), ("forward_tile", ctypes.c_int32),
        ("windows_per_step", ctypes.c_int32),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("steps", ctypes.c_uint64), ("pairs", ctypes.c_uint64), ("word_count_actual", ctypes.c_uint64),
        ("row_bytes", ctypes.c_uint64), ("loss", ctypes.c_double), ("final_alpha", ctypes.c_float),
        ("train_ms", ctypes.c_float), ("workers", ctypes.c_int32), ("warps_per_cta", ctypes.c_int32),
        ("row_loads", ctypes.c_uint64), ("row_stores", ctypes.c_uint64), ("output_rows", ctypes.c_uint64),
        ("forward_tile", ctypes.c_int32), ("warps_per_worker", ctypes.c_int32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class WalkOptions(ctypes.Structure):
    _fields_ = [("walker_num", ctypes.c_int64), ("min_length", ctypes.c_int32), ("max_length", ctypes.c_int32),
                ("r_threshold", ctypes.c_double), ("seed", ctypes.c_uint64), ("trace_steps", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class SgnsError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("sgns status %d: %s" % (status, msg))
        self.status = status


_lib = None


def header_functions():
    """Names of the functions include/sgns.h declares."""
    text = re.sub(r"/\*.*?\*/", " ", open(HEADER).read(), flags=re.S)  # declarations only, not comments
    return sorted(set(re.findall(r"\b(sgns_[a-z_0-9]+)\s*\(", text)))


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libsgns.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        vp, i32, i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
        L.sgns_last_error.restype = ctypes.c_char_p
        L.sgns_last_error.argtypes = [vp]
        L.sgns_default_options.argtypes = [ctypes.POINTER(Options)]
        L.sgns_default_options.restype = None
        L.sgns_options_from_args.argtypes = [ctypes.POINTER(Options), ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
        L.sgns_create.argtypes = [ctypes.POINTER(Options), ctypes.POINTER(vp)]
        L.sgns_destroy.argtypes = [vp]
        L.sgns_destroy.restype = None
        L.sgns_set_vocab.argtypes = [vp, vp, i64]
        L.sgns_reset_model.argtypes = [vp]
        L.sgns_upload_corpus.argtypes = [vp, vp, i64]
        L.sgns_train.argtypes = [vp]
        L.sgns_train_corpus.argtypes = [vp, vp, i64]
        L.sgns_train_walk_files.argtypes = [vp, ctypes.POINTER(ctypes.c_char_p), i32, i64]
        L.sgns_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
        L.sgns_vocab_size.argtypes = [vp]
        L.sgns_vocab_size.restype = i64
        L.sgns_get_order.argtypes = [vp, vp]
        L.sgns_get_embeddings.argtypes = [vp, i32, vp]
        L.sgns_set_embeddings.argtypes = [vp, i32, vp]
        L.sgns_device_tables.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp)]
        L.sgns_save_text.argtypes = [vp, ctypes.c_char_p]
        L.sgns_minibatch_update.argtypes = [i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        L.sgns_minibatch_update_bf16.argtypes = [i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, ctypes.c_uint64, vp]
        L.sgns_minibatch_update_noalloc.argtypes = [i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        L.sgns_parse_walks.argtypes = [vp, i64, vp, i64, ctypes.POINTER(i64), ctypes.POINTER(i64), vp]
        L.sgns_link_scores.argtypes = [i32, i32, vp, i64, vp, i64, vp, vp]
        L.sgns_loss_adjoint.argtypes = [i32, i32, i64, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp,
                                        ctypes.POINTER(i64), vp, vp, ctypes.POINTER(i64), vp]
        L.sgns_edge_common_neighbors.argtypes = [vp, vp, i64, i64, vp, vp]
        L.sgns_info_walks.argtypes = [ctypes.POINTER(WalkOptions), vp, vp, vp, i64, i64, vp, i64,
                                      ctypes.POINTER(i64), vp]
        L.sgns_internal_host_vocab.argtypes = [vp, i64, ctypes.c_float, i64, i32, vp, vp, vp, vp,
                                               ctypes.POINTER(ctypes.c_uint64)]
        L.sgns_internal_host_vocab.restype = i32
        L.sgns_internal_write_embedding.argtypes = [vp, vp, i64, i32, i32, ctypes.c_char_p]
        L.sgns_internal_write_embedding.restype = i32
        L.sgns_sync_rows.argtypes = [vp, ctypes.c_uint64, ctypes.c_uint64, i32, vp, i64, ctypes.POINTER(i64)]
        L.sgns_gather_rows.argtypes = [vp, i32, vp, i64, vp]
        L.sgns_scatter_rows.argtypes = [vp, i32, vp, i64, vp, ctypes.c_float]
        L.sgns_internal_sync_rows.argtypes = [vp, i64, ctypes.c_uint64, ctypes.c_uint64, i32, vp, i64,
                                              ctypes.POINTER(i64)]
        L.sgns_internal_sync_rows.restype = i32
        L.sgns_internal_xlog2x_table.argtypes = [i32, vp]
        L.sgns_internal_xlog2x_table.restype = None
        L.sgns_internal_sr_bits4.argtypes = [i64, vp, vp, vp, vp]
        L.sgns_internal_sr_bits4.restype = None
        for name in header_functions():  # every declared entry point must be exported
            getattr(L, name)
        _lib = L
    return _lib


def _check(status, handle=None):
    if status != OK:
        msg = lib().sgns_last_error(handle)
        raise SgnsError(status, msg.decode() if msg else "")


def default_options(**kw):
    o = Options()
    lib().sgns_default_options(ctypes.byref(o))
    for k, v in kw.items():
        if k == "storage" and isinstance(v, str):
            v = {"fp32": STORE_FP32, "bf16": STORE_BF16_SR}[v]
        if k == "engine" and isinstance(v, str):
            v = {"plain": ENGINE_PLAIN, "persistent": ENGINE_PERSISTENT}[v]
        if k == "mode" and isinstance(v, str):
            v = {"hogwild": MODE_HOGWILD, "exact": MODE_REPLAY_EXACT}[v]
        setattr(o, k, v)
    return o


def options_from_args(args, base=None):
    o = base if base is not None else default_options()
    argv = (ctypes.c_char_p * (len(args) + 1))(*([b"prog"] + [a.encode() for a in args]))
    _check(lib().sgns_options_from_args(ctypes.byref(o), len(args) + 1, argv))
    return o


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


class Trainer:
    """One sgns_handle: vocabulary, device tables, corpus and training calls."""

    def __init__(self, options=None, **kw):
        self.opt = options if options is not None else default_options(**kw)
        h = ctypes.c_void_p()
        _check(lib().sgns_create(ctypes.byref(self.opt), ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().sgns_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_vocab(self, counts):
        counts = np.ascontiguousarray(counts, dtype=np.int32)
        _check(lib().sgns_set_vocab(self.h, _ptr(counts), len(counts)), self.h)

    def reset_model(self):
        _check(lib().sgns_reset_model(self.h), self.h)

    def upload(self, tokens):
        tokens = np.ascontiguousarray(tokens, dtype=np.int32)
        _check(lib().sgns_upload_corpus(self.h, _ptr(tokens), len(tokens)), self.h)

    def train(self):
        _check(lib().sgns_train(self.h), self.h)
        return self.stats()

    def train_corpus(self, tokens):
        """tokens: numpy int32 (host); pinned buffers may be passed as numpy views."""
        tokens = np.ascontiguousarray(tokens, dtype=np.int32)
        _check(lib().sgns_train_corpus(self.h, _ptr(tokens), len(tokens)), self.h)
        return self.stats()

    def train_corpus_ptr(self, ptr, n):
        _check(lib().sgns_train_corpus(self.h, ctypes.c_void_p(ptr), n), self.h)
        return self.stats()

    def train_walk_files(self, paths, vertices=0):
        arr = (ctypes.c_char_p * len(paths))(*[p.encode() for p in paths])
        _check(lib().sgns_train_walk_files(self.h, arr, len(paths), vertices), self.h)
        return self.stats()

    def stats(self):
        s = Stats()
        _check(lib().sgns_get_stats(self.h, ctypes.byref(s)))
        return s

    @property
    def vocab_size(self):
        return lib().sgns_vocab_size(self.h)

    def order(self):
        o = np.zeros(self.vocab_size, dtype=np.uint32)
        _check(lib().sgns_get_order(self.h, _ptr(o)), self.h)
        return o

    def embeddings(self, which=0):
        out = np.zeros((self.vocab_size, self.opt.size), dtype=np.float32)
        _check(lib().sgns_get_embeddings(self.h, which, _ptr(out)), self.h)
        return out

    def embeddings_to(self, which, ptr):
        """sgns_get_embeddings into caller memory at ptr (V * d floats, e.g. a pinned buffer)."""
        _check(lib().sgns_get_embeddings(self.h, which, ctypes.c_void_p(ptr)), self.h)

    def set_embeddings(self, which, values):
        values = np.ascontiguousarray(values, dtype=np.float32)
        _check(lib().sgns_set_embeddings(self.h, which, _ptr(values)), self.h)

    def device_tables(self):
        a, b = ctypes.c_void_p(), ctypes.c_void_p()
        _check(lib().sgns_device_tables(self.h, ctypes.byref(a), ctypes.byref(b)), self.h)
        return a.value, b.value

    def save_text(self, path):
        _check(lib().sgns_save_text(self.h, path.encode()), self.h)

    def sync_rows(self, seed, round, full=False):
        """sgns_sync_rows: the rows of one hotness-block sync round (int32, host)."""
        out = np.zeros(max(self.vocab_size, 1), np.int32)
        n = ctypes.c_int64()
        _check(lib().sgns_sync_rows(self.h, seed, round, int(full), _ptr(out), len(out), ctypes.byref(n)))
        return out[:n.value]

    def gather_rows(self, which, rows, buf):
        """rows: int32 CUDA tensor; buf: float32 CUDA tensor [n, d] (filled)."""
        _check(lib().sgns_gather_rows(self.h, which, rows.data_ptr(), int(rows.numel()), buf.data_ptr()), self.h)

    def scatter_rows(self, which, rows, buf, divisor):
        _check(lib().sgns_scatter_rows(self.h, which, rows.data_ptr(), int(rows.numel()), buf.data_ptr(),
                                       float(divisor)), self.h)

    def sync_hot_rows(self, seed, round, full=False, group=None):
        """One round of the hotness-block sync across the replicas of a torch.distributed
        group (dsgl.hpp:641-756): the round's rows of Wih and Woh, summed over the replicas
        by all_reduce, divided by the replica count."""
        import torch
        import torch.distributed as dist

        rows = torch.from_numpy(self.sync_rows(seed, round, full)).cuda(self.opt.device)
        world = dist.get_world_size(group)
        bufs = {}

        def gather(which, r):
            bufs[which] = torch.empty((r.numel(), self.opt.size), dtype=torch.float32, device=r.device)
            self.gather_rows(which, r, bufs[which])
            return bufs[which]

        hot_row_sync(rows, gather, lambda which, r, b, w: self.scatter_rows(which, r, b, w), world,
                     lambda b: dist.all_reduce(b, op=dist.ReduceOp.SUM, group=group))
        return int(rows.numel())


def minibatch_update(d, in_count, in_first, out_count, out_meta, alpha, in_rows, out_rows, d_in, d_out,
                     stream=0):
    """All array arguments are CUDA torch tensors (device pointers)."""
    n = int(in_count.numel())
    _check(lib().sgns_minibatch_update(d, n, in_count.data_ptr(), in_first.data_ptr(), out_count.data_ptr(),
                                       out_meta.data_ptr(), alpha.data_ptr(), in_rows.data_ptr(),
                                       out_rows.data_ptr(), d_in.data_ptr(), d_out.data_ptr(),
                                       ctypes.c_void_p(stream)))


def minibatch_update_bf16(d, in_count, in_first, out_count, out_meta, alpha, in_rows, out_rows, new_in, new_out,
                          seed, stream=0):
    """sgns_minibatch_update_bf16: the update plus the BF16 trainers' rounded write-back;
    new_in / new_out are int16 (bf16 bits) CUDA tensors shaped like in_rows / out_rows."""
    n = int(in_count.numel())
    _check(lib().sgns_minibatch_update_bf16(d, n, in_count.data_ptr(), in_first.data_ptr(), out_count.data_ptr(),
                                            out_meta.data_ptr(), alpha.data_ptr(), in_rows.data_ptr(),
                                            out_rows.data_ptr(), new_in.data_ptr(), new_out.data_ptr(), int(seed),
                                            ctypes.c_void_p(stream)))


def minibatch_update_noalloc(d, in_count, in_first, out_count, out_meta, alpha, in_rows, out_rows, d_in,
                             d_out, stream=0):
    """sgns_minibatch_update_noalloc: same arguments as minibatch_update, no device allocation."""
    n = int(in_count.numel())
    _check(lib().sgns_minibatch_update_noalloc(d, n, in_count.data_ptr(), in_first.data_ptr(), out_count.data_ptr(),
                                               out_meta.data_ptr(), alpha.data_ptr(), in_rows.data_ptr(),
                                               out_rows.data_ptr(), d_in.data_ptr(), d_out.data_ptr(),
                                               ctypes.c_void_p(stream)))


def parse_walks(text, tokens=None, stream=0):
    """sgns_parse_walks on a uint8 device tensor; tokens: int32 device tensor (None: count
    only).  Returns (n_tokens, max_id)."""
    n_tok, mx = ctypes.c_int64(), ctypes.c_int64()
    cap = int(tokens.numel()) if tokens is not None else 0
    _check(lib().sgns_parse_walks(text.data_ptr() if text.numel() else None, int(text.numel()),
                                  tokens.data_ptr() if tokens is not None else None, cap, ctypes.byref(n_tok),
                                  ctypes.byref(mx), ctypes.c_void_p(stream)))
    return n_tok.value, mx.value


def parse_walks_count(text, stream=0):
    """Number of tokens the walk text yields (the capacity error carries it)."""
    n_tok, mx = ctypes.c_int64(), ctypes.c_int64()
    st = lib().sgns_parse_walks(text.data_ptr() if text.numel() else None, int(text.numel()), None, 0,
                                ctypes.byref(n_tok), ctypes.byref(mx), ctypes.c_void_p(stream))
    if st not in (OK, EINVAL) or (st == EINVAL and n_tok.value == 0):
        _check(st)
    return n_tok.value


def link_scores(dtype, d, table, V, pairs, scores, stream=0):
    """sgns_link_scores: table is a device pointer (int) or tensor of V x d (fp32 or bf16
    bits), pairs an int32 device tensor of shape [n, 2] (row indices), scores a float32
    device tensor of n entries."""
    tp = table if isinstance(table, int) else table.data_ptr()
    _check(lib().sgns_link_scores(dtype, d, ctypes.c_void_p(tp), V, pairs.data_ptr(), int(pairs.shape[0]),
                                  scores.data_ptr(), ctypes.c_void_p(stream)))


def loss_adjoint(dtype, d, V, in_ptr, in_ids, in_first, out_ptr, out_ids, out_meta, wih, woh, loss,
                 grad_in_ids, grad_in, grad_out_ids, grad_out, stream=0):
    """Device tensors in, (n_in, n_out) out; fills loss / ids / grads in place."""
    n = int(in_first.numel())
    n_in, n_out = ctypes.c_int64(), ctypes.c_int64()
    _check(lib().sgns_loss_adjoint(dtype, d, V, n, in_ptr.data_ptr(), in_ids.data_ptr(), in_first.data_ptr(),
                                   out_ptr.data_ptr(), out_ids.data_ptr(), out_meta.data_ptr(), wih, woh,
                                   loss.data_ptr(), grad_in_ids.data_ptr(), grad_in.data_ptr(),
                                   ctypes.byref(n_in), grad_out_ids.data_ptr(), grad_out.data_ptr(),
                                   ctypes.byref(n_out), ctypes.c_void_p(stream)))
    return n_in.value, n_out.value


def edge_common_neighbors(indptr, indices, cn, stream=0):
    """sgns_edge_common_neighbors on device tensors (indptr int64 [V + 1], indices int32 [E],
    cn int32 [E], filled in place)."""
    V, E = int(indptr.numel()) - 1, int(indices.numel())
    _check(lib().sgns_edge_common_neighbors(indptr.data_ptr(), indices.data_ptr() if E else None, V, E,
                                            cn.data_ptr() if E else None, ctypes.c_void_p(stream)))


def info_walks(indptr, indices, cn, walker_num, min_length=20, max_length=80, r_threshold=0.999, seed=1,
               corpus=None, stream=0, trace=1):
    """sgns_info_walks on device tensors.  corpus: int32 device tensor to fill (None: a new
    one of the exact size, after a counting call).  Returns (corpus, n_tokens)."""
    import torch

    V, E = int(indptr.numel()) - 1, int(indices.numel())
    o = WalkOptions(walker_num=int(walker_num), min_length=int(min_length), max_length=int(max_length),
                    r_threshold=float(r_threshold), seed=int(seed), trace_steps=int(trace))
    n = ctypes.c_int64()
    args = (indptr.data_ptr(), indices.data_ptr() if E else None, cn.data_ptr() if E else None, V, E)
    if corpus is None:
        _check(lib().sgns_info_walks(ctypes.byref(o), *args, None, 0, ctypes.byref(n), ctypes.c_void_p(stream)))
        corpus = torch.empty(max(n.value, 1), dtype=torch.int32, device=indptr.device)
    _check(lib().sgns_info_walks(ctypes.byref(o), *args, corpus.data_ptr(), int(corpus.numel()), ctypes.byref(n),
                                 ctypes.c_void_p(stream)))
    return corpus[:n.value], n.value


def hot_row_sync(rows, gather, scatter, world, all_reduce):
    """The exchange of one hotness-block sync round (dsgl.hpp:731-755), for any transport:
    for Wih then Woh, gather(which, rows) -> rows as an fp32 buffer, all_reduce(buffer)
    sums it over the replicas in place, scatter(which, rows, buffer, world) stores
    buffer / world back."""
    for which in (0, 1):
        buf = gather(which, rows)
        all_reduce(buf)
        scatter(which, rows, buf, float(world))


def internal_sync_rows(cn_sorted, seed, round, full=False):
    """The row draw of sgns_sync_rows from count-sorted counts, on the host (no device)."""
    cn_sorted = np.ascontiguousarray(cn_sorted, dtype=np.int32)
    out = np.zeros(max(len(cn_sorted), 1), np.int32)
    n = ctypes.c_int64()
    _check(lib().sgns_internal_sync_rows(_ptr(cn_sorted), len(cn_sorted), seed, round, int(full), _ptr(out), len(out),
                                         ctypes.byref(n)))
    return out[:n.value]


def host_vocab(counts, sample, table_size, threads):
    """The host set-up sgns_set_vocab performs, run on the CPU without a device: (order of the
    count-sorted rows, unigram table, subsampling keep thresholds, sigmoid table,
    train_words)."""
    counts = np.ascontiguousarray(counts, dtype=np.int32)
    V = len(counts)
    order = np.zeros(V, np.uint32)
    table = np.zeros(table_size, np.int32)
    ran = np.zeros(V, np.float32)
    exp = np.zeros(1001, np.float32)
    tw = ctypes.c_uint64()
    _check(lib().sgns_internal_host_vocab(_ptr(counts), V, sample, table_size, threads, _ptr(order), _ptr(table),
                                          _ptr(ran), _ptr(exp), ctypes.byref(tw)))
    return order, table, ran, exp, tw.value


def write_embedding(order, w, path, binary=False):
    """The writer of sgns_save_text on host arrays (order: V row ids, w: V x d floats in
    sorted-row order), run on the CPU without a device."""
    order = np.ascontiguousarray(order, dtype=np.uint32)
    w = np.ascontiguousarray(w, dtype=np.float32)
    _check(lib().sgns_internal_write_embedding(_ptr(order), _ptr(w), w.shape[0], w.shape[1], int(binary),
                                               str(path).encode()))


def xlog2x_table(n):
    """The walker's x * log2(x) table as sgns_info_walks builds it (host code, no device)."""
    t = np.zeros(n, np.float64)
    lib().sgns_internal_xlog2x_table(n, _ptr(t))
    return t


def sr_bits4(ev, row, col4):
    """The stochastic-rounding bits (uint64 per triple) the kernels draw for column chunk
    col4 of row `row` under event key ev (host copy of the device function, no device)."""
    ev = np.ascontiguousarray(ev, np.uint64)
    row = np.ascontiguousarray(row, np.uint32)
    col4 = np.ascontiguousarray(col4, np.uint32)
    out = np.zeros(len(ev), np.uint64)
    lib().sgns_internal_sr_bits4(len(ev), _ptr(ev), _ptr(row), _ptr(col4), _ptr(out))
    return out
