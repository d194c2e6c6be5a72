"""The C ABI library without a GPU: symbols, option parsing, arithmetic helpers."""
import ctypes
import os
import random
import subprocess

import numpy as np
import pytest

import sgns


def test_every_declared_symbol_is_exported(sgns_lib):
    names = sgns.header_functions()
    assert len(names) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", sgns.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in names if n not in exported]
    assert not missing, missing




@pytest.mark.parametrize("cmd", [["gcc", "-std=c99", "-x", "c"], ["g++", "-std=c++11", "-x", "c++"]])
def test_header_compiles_alone(cmd, tmp_path):
    """include/sgns.h is self-contained and warning-free as C99 and as C++11, the languages
    of the callers it replaces (the reference builds its trainer as C++)."""
    src = tmp_path / "inc.txt"
    src.write_text('#include "sgns.h"\n')
    subprocess.run(cmd + ["-pedantic", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I",
                          os.path.dirname(sgns.HEADER), str(src)], check=True)

@pytest.mark.parametrize("ctype,cname", [(sgns.Options, "sgns_options"), (sgns.Stats, "sgns_stats")])
def test_ctypes_structs_match_the_header(ctype, cname, tmp_path):
    """The binding's struct mirrors have the C layout of include/sgns.h: size and the
    offset of every field, as a C compiler lays them out."""
    fields = [f for f, _ in ctype._fields_]
    src = tmp_path / "layout.c"
    src.write_text("#include <stddef.h>\n#include <stdio.h>\n#include \"sgns.h\"\nint main(void) {\n"
                   + '  printf("%%zu\\n", sizeof(%s));\n' % cname
                   + "".join('  printf("%%zu\\n", offsetof(%s, %s));\n' % (cname, f) for f in fields)
                   + "  return 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.dirname(sgns.HEADER), str(src), "-o", str(exe)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert out[0] == ctypes.sizeof(ctype)
    assert out[1:] == [getattr(ctype, f).offset for f in fields]

def test_defaults_are_the_references(sgns_lib):
    o = sgns.default_options()
    # include/dsgl.hpp:67-76, 82
    assert (o.size, o.window, o.negative, o.iter, o.threads, o.batch_size, o.min_count) == (100, 5, 5, 5, 12, 11, 5)
    assert abs(o.alpha - 0.1) < 1e-7 and abs(o.sample - 1e-3) < 1e-9
    assert o.table_size == 100000000


def test_reference_flags_parse(sgns_lib):
    args = ["-size", "128", "-window", "10", "-negative", "5", "-batch-size", "21", "-sample", "1e-3",
            "-alpha", "0.01", "-min-count", "0", "-iter", "3", "-threads", "10", "-debug", "2",
            "-sync-size", "1024", "-storage", "bf16", "-engine", "plain", "-workers", "77"]
    o = sgns.options_from_args(args)
    assert (o.size, o.window, o.negative, o.batch_size, o.min_count, o.iter, o.threads) == (128, 10, 5, 21, 0, 3, 10)
    assert abs(o.alpha - 0.01) < 1e-8
    assert o.storage == sgns.STORE_BF16_SR and o.engine == sgns.ENGINE_PLAIN and o.workers == 77


def test_flag_without_value_is_an_error(sgns_lib):
    with pytest.raises(sgns.SgnsError) as e:
        sgns.options_from_args(["-size"])
    assert e.value.status == sgns.EINVAL


def test_bad_storage_name(sgns_lib):
    with pytest.raises(sgns.SgnsError):
        sgns.options_from_args(["-storage", "fp8"])


def test_mode_flag(sgns_lib):
    assert sgns.default_options().mode == sgns.MODE_HOGWILD
    assert sgns.options_from_args(["-mode", "exact"]).mode == sgns.MODE_REPLAY_EXACT
    assert sgns.options_from_args(["-mode", "hogwild"]).mode == sgns.MODE_HOGWILD
    with pytest.raises(sgns.SgnsError) as e:
        sgns.options_from_args(["-mode", "lockstep"])
    assert e.value.status == sgns.EINVAL


def test_invalid_options_rejected_before_device(sgns_lib):
    for kw in (dict(size=130), dict(size=512), dict(window=0), dict(window=16), dict(negative=11), dict(iter=0),
               dict(mode=2), dict(mode="exact", workers=2)):
        with pytest.raises(sgns.SgnsError) as e:
            sgns.Trainer(**kw)
        assert e.value.status == sgns.EINVAL


def test_create_without_gpu_fails_loudly(sgns_lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(sgns.SgnsError) as e:
        sgns.Trainer(size=16)
    assert e.value.status == sgns.ECUDA


def test_kernel_level_entry_points_check_arguments_first(sgns_lib):
    """Bad arguments are rejected with SGNS_EINVAL before any device is touched."""
    import ctypes

    L = sgns.lib()
    n_tok, mx = ctypes.c_int64(), ctypes.c_int64()
    # walk-text parse: null text of nonzero size, negative size, capacity without a buffer
    assert L.sgns_parse_walks(None, 5, None, 0, ctypes.byref(n_tok), ctypes.byref(mx), None) == sgns.EINVAL
    assert L.sgns_parse_walks(None, -1, None, 0, ctypes.byref(n_tok), ctypes.byref(mx), None) == sgns.EINVAL
    fake = ctypes.c_void_p(16)  # never dereferenced: the call fails on the missing output
    assert L.sgns_parse_walks(fake, 4, None, 8, ctypes.byref(n_tok), ctypes.byref(mx), None) == sgns.EINVAL
    # link scores: unknown dtype, d not a multiple of 4, d too large, missing buffers
    for args in ((2, 8, fake, 10, fake, 1, fake), (0, 6, fake, 10, fake, 1, fake),
                 (0, 512, fake, 10, fake, 1, fake), (0, 8, None, 10, fake, 1, fake)):
        assert L.sgns_link_scores(*args, None) == sgns.EINVAL
    assert b"link-score" in L.sgns_last_error(None)
    assert L.sgns_link_scores(0, 8, fake, 10, fake, 0, fake, None) == sgns.OK  # nothing to do


def test_handle_less_errors_are_per_thread(sgns_lib):
    """sgns_last_error(NULL) reports the calling thread's own last failure."""
    import ctypes
    import threading

    L = sgns.lib()
    n_tok, mx = ctypes.c_int64(), ctypes.c_int64()
    seen = {}
    both_failed = threading.Barrier(2)

    def worker(name, fn):
        assert fn() == sgns.EINVAL
        both_failed.wait()  # the other thread has failed too before either reads
        seen[name] = L.sgns_last_error(None)

    fake = ctypes.c_void_p(16)
    t1 = threading.Thread(target=worker, args=("parse", lambda: L.sgns_parse_walks(
        None, 5, None, 0, ctypes.byref(n_tok), ctypes.byref(mx), None)))
    t2 = threading.Thread(target=worker, args=("score", lambda: L.sgns_link_scores(
        7, 8, fake, 10, fake, 1, fake, None)))
    for t in (t1, t2):
        t.start()
    for t in (t1, t2):
        t.join()
    assert b"walk-parse" in seen["parse"] and b"link-score" in seen["score"]


def test_command_line_wildcard_without_match_is_an_error(sgns_lib, tmp_path):
    import os

    cli = os.path.join(os.path.dirname(sgns.LIB_PATH), "sgns_train")
    r = subprocess.run([cli, "-train", str(tmp_path / "walks-*.txt")], capture_output=True, text=True)
    assert r.returncode == 1 and "no walk file matches" in r.stderr


def test_walk_text_formatter_writes_the_reference_format():
    """bench.format_walk_text (the text the ingest benchmark parses) is the reference's
    walk format, byte for byte as synth.write_walk_file writes it."""
    import os
    import sys
    import tempfile
    import torch

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    import synth

    rng = np.random.default_rng(8)
    walks = [rng.integers(0, 2**31 - 1 if k % 5 == 0 else 100000, size=rng.integers(1, 30)) for k in range(200)]
    corpus = np.concatenate([np.append(w, -1) for w in walks]).astype(np.int32)
    text = bench.format_walk_text(torch.from_numpy(corpus)).numpy().tobytes()
    path = os.path.join(tempfile.mkdtemp(), "w.txt")
    synth.write_walk_file(corpus, path)
    assert text == open(path, "rb").read()


# ---- arithmetic the kernels rely on, restated exactly in Python ---------------------
def gm_magic(d):
    l = 0
    while (1 << l) < d:
        l += 1
    m = ((1 << 64) * ((1 << l) - d)) // d + 1
    return m & ((1 << 64) - 1), l - 1


def gm_div(n, d):
    if d == 1:
        return n
    m, sh = gm_magic(d)
    t = (m * n) >> 64
    return (t + ((n - t) >> 1)) >> sh


@pytest.mark.parametrize("d", [2, 3, 5, 7, 10, 1099, 1500, 9999, 10_000_000, 100_000_000, 2_238_730, 3_999_999,
                               (1 << 31) - 1, (1 << 32) + 15, (1 << 63) + 12345])
def test_invariant_division(d):
    rnd = random.Random(d)
    vals = [0, 1, d - 1, d, d + 1, 2 * d - 1, (1 << 48) - 1, (1 << 64) - 1, (1 << 63)]
    vals += [rnd.getrandbits(64) for _ in range(2000)] + [rnd.getrandbits(48) for _ in range(2000)]
    for n in vals:
        assert gm_div(n, d) == n // d


def test_lcg_jump_ahead():
    A, C, M = 25214903917, 11, (1 << 64) - 1
    pm, pa = A, C
    pows = []
    for _ in range(20):
        pows.append((pm, pa))
        pa = (pm * pa + pa) & M
        pm = (pm * pm) & M
    r0 = 12345
    for n in (0, 1, 2, 31, 32, 33, 1000, 65537):
        r = r0
        for _ in range(n):
            r = (r * A + C) & M
        j, k, i = r0, n, 0
        while k:
            if k & 1:
                j = (pows[i][0] * j + pows[i][1]) & M
            k >>= 1
            i += 1
        assert j == r


def test_bf16_stochastic_rounding_is_unbiased():
    # the rounding rule of the kernels and the oracle: add 16 uniform bits, truncate
    rng = np.random.default_rng(0)
    x = np.float32(1.0 + 2 ** -9 * 0.3)
    u = np.array([x], np.float32).view(np.uint32)[0]
    r = rng.integers(0, 1 << 16, 200000).astype(np.uint64)
    v = ((np.uint64(u) + r) >> np.uint64(16)).astype(np.uint32) << 16
    mean = v.view(np.float32).astype(np.float64).mean()
    assert abs(mean - float(x)) < 2 ** -9 * 0.01


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_host_vocabulary_setup_equals_the_oracle(seed, sgns_lib, oracle_mod):
    """The library's host set-up of a vocabulary (what sgns_set_vocab uploads) against the
    oracle: row order under std::sort with many tied counts and zero counts, the unigram
    table, the sigmoid table bit for bit; the keep thresholds against a float32
    restatement of dsgl.hpp:923-924 (sqrt(r) + r, r = sample * train_words / count)."""
    rng = np.random.default_rng(seed)
    V = int(rng.integers(1001, 5000))
    counts = np.minimum(rng.zipf(1.6, V), 5000).astype(np.int32) - (rng.random(V) < 0.05).astype(np.int32)
    sample, table_size, threads = [1e-3, 1e-4, 0.0][seed], int(rng.integers(10_000, 300_000)), [1, 4, 12][seed]
    order, table, ran, exp, tw = sgns.host_vocab(counts, sample, table_size, threads)
    o_order, _, o_cns, o_tw = oracle_mod.vocab(counts)
    assert tw == o_tw == int(counts.sum())
    assert np.array_equal(order, o_order)
    assert np.array_equal(table, oracle_mod.unigram_table(o_cns, table_size, threads))
    assert np.array_equal(exp.view(np.uint32), oracle_mod.exp_table().view(np.uint32))
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.float32(sample) * np.float32(tw) / counts.astype(np.float32)
        want = np.sqrt(r) + r
    want = want.astype(np.float32)
    nan = np.isnan(want)  # 0/0 for a zero count with sample 0: compared as NaN, not by bits
    assert np.array_equal(np.isnan(ran), nan)
    assert np.array_equal(ran[~nan].view(np.uint32), want[~nan].view(np.uint32))


def test_host_vocabulary_setup_rejects_bad_input(sgns_lib):
    with pytest.raises(sgns.SgnsError):
        sgns.host_vocab(np.array([3, -1, 2], np.int32), 1e-3, 100, 1)
    with pytest.raises(sgns.SgnsError):
        sgns.host_vocab(np.array([3, 1, 2], np.int32), 1e-3, 0, 1)
