"""Full-size check of the persistent engine on the headline workload.

The trainer's control flow (corpus slices, subsampling, window draws, negative pools, walk
pairing and flushes) depends only on the corpus, the configuration and the worker count,
never on the table values or on d (include/dsgl.hpp:811-1407: every branch reads the
corpus, the LCG or the counts).  So the oracle at d = 4, given the GPU run's worker count,
reproduces the exact step, pair and word counts of a full-size BF16 training pass of the
LiveJournal-sized Chung-Lu workload (797.6 M tokens, 7.6 G pairs, 1064 workers) in one to
two minutes on the host cores.  The counts are integers: they must be equal."""
import os

import numpy as np
import pytest

import sgns

pytestmark = pytest.mark.gpu


def test_full_size_control_flow_equals_the_oracle(sgns_lib, oracle_mod):
    import torch

    import bench

    wl = bench.WORKLOADS["lj-cl"]
    corpus, _, _, _, _ = bench.make_corpus(wl, 0, torch.device("cuda", 0))
    c = np.ascontiguousarray(corpus.cpu().numpy(), dtype=np.int32)
    del corpus
    torch.cuda.empty_cache()
    counts = np.bincount(c[c >= 0], minlength=wl["V"]).astype(np.int32)
    tr = bench.TRAIN
    opt = sgns.default_options(iter=1, storage="bf16", engine="persistent", device=0, debug=0, warps_per_cta=7,
                               **tr)
    with sgns.Trainer(opt) as t:
        t.set_vocab(counts)
        st = t.train_corpus(c)
        wih = t.embeddings(0)
    assert np.isfinite(wih).all() and float(np.abs(wih).max()) > 0
    _, _, ost = oracle_mod.train(c, counts, d=4, window=tr["window"], negative=tr["negative"], iter=1,
                                 workers=st.workers, threads=len(os.sched_getaffinity(0)),
                                 table_threads=tr["threads"],
                                 policy=oracle_mod.POLICY_WINDOW, storage=oracle_mod.STORE_F32,
                                 table_size=tr["table_size"], sample=tr["sample"], alpha=tr["alpha"])
    assert st.word_count_actual == len(c)
    assert (st.steps, st.pairs, st.word_count_actual) == (ost["steps"], ost["pairs"], ost["word_count_actual"])
