"""Differential check of the oracle against the reference's own trainer on fresh random
configurations (beyond the fixed golden cases).

The reference binary (oracle/_ref/dsgl_ref) is compiled from the reference checkout by
oracle/build_ref.sh where that checkout exists; elsewhere these tests are skipped.  One
compute thread (-threads 2) makes the reference deterministic; the oracle then must give
the same vocabulary order and the same Wih and Woh bit for bit.

The configurations and corpora come from tests/random_configs.py (which also explains
why it breaks ties of the largest count: they crash the reference).
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from random_configs import random_case

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "dsgl_ref")

pytestmark = pytest.mark.skipif(not os.path.exists(REF_BIN), reason="reference binary not built here")


@pytest.mark.parametrize("seed", [19, 26, 101, 202, 303, 404, 1000, 1001, 1002, 1003])
def test_oracle_equals_reference_on_random_configs(seed, oracle_mod):
    cfg, corpus = random_case(seed)
    V, d = cfg["V"], cfg["d"]
    with tempfile.TemporaryDirectory() as tmp:
        cpath = os.path.join(tmp, "c.i32")
        corpus.tofile(cpath)
        pre = os.path.join(tmp, "r")
        flags = ["-size", str(d), "-window", str(cfg["window"]), "-negative", str(cfg["negative"]),
                 "-iter", str(cfg["iter"]), "-sample", repr(cfg["sample"]), "-alpha", repr(cfg["alpha"]),
                 "-threads", "2", "-debug", "0", "-eoutput", pre + ".txt"]  # the reference always saves
        r = subprocess.run([REF_BIN, cpath, str(V), pre] + flags, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, (r.returncode, r.stderr[-2000:])
        rwih = np.fromfile(pre + ".wih", dtype=np.float32).reshape(V, d)
        rwoh = np.fromfile(pre + ".woh", dtype=np.float32).reshape(V, d)
        rorder = np.fromfile(pre + ".order", dtype=np.uint32)
    counts = np.bincount(corpus[corpus >= 0], minlength=V).astype(np.int32)
    order, _, _, _ = oracle_mod.vocab(counts)
    wih, woh, _ = oracle_mod.train(corpus, counts, d=d, window=cfg["window"], negative=cfg["negative"],
                                   iter=cfg["iter"], workers=1, threads=1, table_threads=2,
                                   policy=oracle_mod.POLICY_REF, storage=oracle_mod.STORE_F32,
                                   table_size=100_000_000, sample=cfg["sample"], alpha=cfg["alpha"])
    assert np.array_equal(np.asarray(order, dtype=np.uint32), rorder)
    assert np.array_equal(wih.view(np.uint32), rwih.view(np.uint32)), np.abs(wih - rwih).max()
    assert np.array_equal(woh.view(np.uint32), rwoh.view(np.uint32)), np.abs(woh - rwoh).max()
