"""Configuration 1 at its stated size: a seeded Chung-Lu graph of 10,000 vertices and
about 100,000 edges (exponent 2.1), 10 uniform random walks of length 80 per vertex
(8 million tokens), d = 128, window 10, 5 negatives, batch 21, sample 1e-3, alpha 0.01
with linear decay, one pass, a 1e7-entry unigram table.  Replay-exact mode (one worker,
the reference's single-compute-thread order) must equal the oracle bit for bit: the plain
engine against the reference buffer policy, the persistent engine against the window
policy, in fp32 and bf16.

The three oracle runs (minutes of single-thread work each) start first, in parallel child
processes (spawned, so no CUDA state is inherited), while the GPU trains."""
import concurrent.futures as cf
import hashlib
import multiprocessing as mp
import os
import sys

import numpy as np
import pytest

from test_gpu_parity import gpu_train

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CFG = dict(V=10000, d=128, window=10, negative=5, iter=1, sample=1e-3, alpha=0.01)
TABLE = 10_000_000
RUNS = [("plain", "fp32", 0), ("persistent", "fp32", 1), ("persistent", "bf16", 1)]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def oracle_job(path, policy, storage):
    """Child process: the oracle on the saved corpus; returns digests and counts."""
    for p in (os.path.join(ROOT, "oracle"), os.path.join(ROOT, "gdistger-re_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import oracle

    corpus = np.load(path)
    counts = np.bincount(corpus[corpus >= 0], minlength=CFG["V"]).astype(np.int32)
    st = {"fp32": oracle.STORE_F32, "bf16": oracle.STORE_BF16}[storage]
    wih, woh, stats = oracle.train(corpus, counts, d=CFG["d"], window=CFG["window"], negative=CFG["negative"],
                                   iter=CFG["iter"], workers=1, threads=1, table_threads=2, policy=policy, storage=st,
                                   table_size=TABLE, sample=CFG["sample"], alpha=CFG["alpha"])
    if storage == "bf16":
        wih, woh = oracle.bf16_to_f32(wih), oracle.bf16_to_f32(woh)
    return sha(wih.astype(np.float32)), sha(woh.astype(np.float32)), (stats["steps"], stats["pairs"],
                                                                      stats["word_count_actual"])


@pytest.fixture(scope="module")
def config1_oracle(tmp_path_factory):
    import synth

    ip, ix = synth.chung_lu(10000, 100000, 2.1, seed=1001)
    corpus = synth.random_walks(ip, ix, 10, 80, seed=1002).numpy().astype(np.int32)
    path = str(tmp_path_factory.mktemp("config1") / "corpus.npy")
    np.save(path, corpus)
    ex = cf.ProcessPoolExecutor(max_workers=len(RUNS), mp_context=mp.get_context("spawn"))
    futures = {(e, s): ex.submit(oracle_job, path, pol, s) for e, s, pol in RUNS}
    yield corpus, futures
    ex.shutdown(wait=True)


@pytest.mark.parametrize("engine,storage", [(e, s) for e, s, _ in RUNS])
def test_config1_replay_exact_equals_oracle(engine, storage, config1_oracle, sgns_lib):
    corpus, futures = config1_oracle
    # 10 walks per vertex, each closed by -1; 80 vertices long except from isolated vertices
    assert (corpus == -1).sum() == 100000 and len(corpus) > 8_000_000
    wih, woh, st, _ = gpu_train(CFG, corpus, engine, storage, workers=0, wpc=0, table_size=TABLE, mode="exact")
    owih_sha, owoh_sha, counts = futures[(engine, storage)].result(timeout=1800)
    assert st.workers == 1
    assert (st.steps, st.pairs, st.word_count_actual) == counts
    assert sha(wih) == owih_sha
    assert sha(woh) == owoh_sha
