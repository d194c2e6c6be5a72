"""The oracle against the reference's own outputs (tests/golden/, made by
tests/golden/make_golden.py from the unmodified include/dsgl.hpp)."""
import glob
import hashlib
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# the reference-output cases: a .json (flags, digests) with its .npz (corpus, rows)
CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(name):
    meta = json.load(open(os.path.join(GOLDEN, name + ".json")))
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return meta, z["corpus"], z["order"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_cases_present():
    assert len(CASES) >= 5


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_bit_for_bit(name, oracle_mod):
    meta, corpus, order = load(name)
    counts = np.bincount(corpus[corpus >= 0], minlength=meta["V"]).astype(np.int32)
    wih, woh, st = oracle_mod.train(corpus, counts, d=meta["d"], window=meta["window"],
                                    negative=meta["negative"], iter=meta["iter"], workers=1, threads=1,
                                    table_threads=meta["table_threads"], policy=oracle_mod.POLICY_REF,
                                    storage=oracle_mod.STORE_F32, table_size=meta["table_size"],
                                    sample=meta["sample"], alpha=meta["alpha"])
    o, _, _, _ = oracle_mod.vocab(counts)
    assert np.array_equal(o, order)
    assert sha(wih) == meta["wih_sha256"], np.abs(wih[0] - np.array(meta["wih_row0"], np.float32)).max()
    assert sha(woh) == meta["woh_sha256"]
    assert st["steps"] > 0


def test_sigmoid_table_matches_reference(oracle_mod):
    meta, _, _ = load(CASES[0])
    assert sha(oracle_mod.exp_table()) == meta["exp_sha256"]


@pytest.mark.parametrize("name", CASES[:2])
def test_unigram_table_matches_reference(name, oracle_mod):
    meta, corpus, _ = load(name)
    counts = np.bincount(corpus[corpus >= 0], minlength=meta["V"]).astype(np.int32)
    _, _, cns, _ = oracle_mod.vocab(counts)
    t = oracle_mod.unigram_table(cns, meta["table_size"], meta["table_threads"])
    assert sha(t) == meta["table_sha256"]


def test_init_matches_reference_lcg(oracle_mod):
    # dsgl.hpp:451-456 restated independently in Python
    V, d = 3, 4
    w = oracle_mod.init_wih(V, d).reshape(-1)
    r = 1
    for i in range(V * d):
        r = (r * 25214903917 + 11) % (1 << 64)
        v = np.float32((np.float32(r & 0xFFFF) / np.float32(65536.0)) - np.float32(0.5)) / np.float32(d)
        assert w[i] == np.float32(v)


@pytest.mark.parametrize("policy", [0, 1])
@pytest.mark.parametrize("name", ["basic", "d128_w10"])
def test_control_flow_does_not_depend_on_d(name, policy, oracle_mod):
    """Steps, pairs and word counts depend on the corpus, the configuration and the worker
    count, not on the table values or d: the premise of the full-size GPU check, which
    counts with the oracle at d = 4.  Many Hogwild workers on several threads."""
    meta, corpus, _ = load(name)
    counts = np.bincount(corpus[corpus >= 0], minlength=meta["V"]).astype(np.int32)
    runs = []
    for d, storage in ((4, oracle_mod.STORE_F32), (meta["d"], oracle_mod.STORE_F32), (64, oracle_mod.STORE_BF16)):
        _, _, st = oracle_mod.train(corpus, counts, d=d, window=meta["window"], negative=meta["negative"],
                                    iter=meta["iter"], workers=23, threads=4, table_threads=meta["table_threads"],
                                    policy=policy, storage=storage, table_size=meta["table_size"],
                                    sample=meta["sample"], alpha=meta["alpha"])
        runs.append((st["steps"], st["pairs"], st["word_count_actual"]))
    assert runs[0][0] > 0 and runs[0] == runs[1] == runs[2], runs


@pytest.mark.parametrize("name", CASES)
def test_embedding_writer_reproduces_reference_file(name, sgns_lib, oracle_mod, tmp_path):
    """The library's writer of sgns_save_text (my_saveModel, dsgl.hpp:1443-1461), fed the
    oracle's Wih (equal to the reference's bit for bit), writes the reference's own -eoutput
    file byte for byte; binary mode writes the raw floats after each id."""
    import sgns

    meta, corpus, _ = load(name)
    counts = np.bincount(corpus[corpus >= 0], minlength=meta["V"]).astype(np.int32)
    wih, _, _ = oracle_mod.train(corpus, counts, d=meta["d"], window=meta["window"], negative=meta["negative"],
                                 iter=meta["iter"], workers=1, threads=1, table_threads=meta["table_threads"],
                                 policy=oracle_mod.POLICY_REF, storage=oracle_mod.STORE_F32,
                                 table_size=meta["table_size"], sample=meta["sample"], alpha=meta["alpha"])
    order, _, _, _ = oracle_mod.vocab(counts)
    out = tmp_path / "emb.txt"
    sgns.write_embedding(order, wih, out)
    assert hashlib.sha256(out.read_bytes()).hexdigest() == meta["text_sha256"]
    sgns.write_embedding(order, wih, out, binary=True)
    raw = out.read_bytes()
    head = b"%d %d\n" % wih.shape
    assert raw.startswith(head)
    pos, d = len(head), wih.shape[1]
    for r in (0, len(order) - 1):  # first and last rows
        if r:
            pos = len(raw) - (len(b"%u " % order[r]) + 4 * d + 1)
        ident = b"%u " % order[r]
        assert raw[pos:pos + len(ident)] == ident
        row = np.frombuffer(raw[pos + len(ident):pos + len(ident) + 4 * d], np.float32)
        assert np.array_equal(row.view(np.uint32), wih[r].view(np.uint32))


@pytest.mark.parametrize("policy", [0, 1])
def test_round_robin_schedule_keeps_the_control_flow(policy, oracle_mod):
    """The schedule that keeps every worker in flight (the oracle's model of a GPU's
    concurrency) trains the same steps, pairs and words as workers run to completion."""
    meta, corpus, _ = load("d128_w10")
    counts = np.bincount(corpus[corpus >= 0], minlength=meta["V"]).astype(np.int32)
    runs = []
    for schedule, threads in ((0, 1), (1, 1), (1, 3)):
        _, _, st = oracle_mod.train(corpus, counts, d=8, window=meta["window"], negative=meta["negative"],
                                    iter=meta["iter"], workers=17, threads=threads, table_threads=meta["table_threads"],
                                    policy=policy, storage=oracle_mod.STORE_F32, table_size=meta["table_size"],
                                    sample=meta["sample"], alpha=meta["alpha"], schedule=schedule)
        runs.append((st["steps"], st["pairs"], st["word_count_actual"]))
    assert runs[0][0] > 0 and runs[0] == runs[1] == runs[2], runs


def test_single_window_step_count(oracle_mod):
    """windows_per_step = 1 without subsampling: one step per position of every walk of
    length > 1 except the pass's last walk, which the reference discards unflushed when the
    slice ends (dsgl.hpp:1031-1050)."""
    rng = np.random.default_rng(4)
    walks = [rng.integers(0, 1200, rng.integers(1, 40)).tolist() for _ in range(300)]
    corpus = np.array([t for w in walks for t in w + [-1]], np.int32)
    counts = np.bincount(corpus[corpus >= 0], minlength=1200).astype(np.int32)
    _, _, st = oracle_mod.train(corpus, counts, d=8, window=3, negative=4, iter=1, workers=1, threads=1,
                                table_threads=2, table_size=100000, sample=0.0, windows=1)
    kept = [len(w) for w in walks if len(w) > 1]
    assert st["steps"] == sum(kept[:-1])
