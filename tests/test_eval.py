"""Link-prediction scoring (sgns_link_scores): the GPU scores of held-out pairs against the
oracle's restatement of the same fixed summation order, and the AUC built on them."""
import numpy as np
import pytest

import sgns


def test_oracle_scores_are_dot_products(oracle_mod):
    rng = np.random.default_rng(3)
    for d in (4, 12, 100, 128, 256):
        t = rng.standard_normal((40, d)).astype(np.float32)
        pr = rng.integers(0, 40, size=(300, 2)).astype(np.int32)
        sc, bad = oracle_mod.link_scores(t, pr)
        ref = (t[pr[:, 0]].astype(np.float64) * t[pr[:, 1]]).sum(1)
        assert not bad and np.allclose(sc, ref, rtol=1e-5, atol=1e-5 * np.abs(ref).max())
    sc, bad = oracle_mod.link_scores(t, np.array([[0, 40], [1, 2]], np.int32))
    assert bad and sc[0] == 0.0


def test_auc_from_scores_matches_pairwise_count():
    import torch
    import synth

    rng = np.random.default_rng(4)
    sp = torch.tensor(rng.normal(0.5, 1.0, 300).round(1), dtype=torch.float32)  # with ties
    sn = torch.tensor(rng.normal(0.0, 1.0, 200).round(1), dtype=torch.float32)
    wins = (sp[:, None] > sn[None, :]).double().sum() + 0.5 * (sp[:, None] == sn[None, :]).double().sum()
    assert abs(synth.auc_from_scores(sp, sn) - float(wins) / (300 * 200)) < 1e-12


@pytest.mark.gpu
def test_gpu_scores_match_oracle(sgns_lib, oracle_mod):
    import torch

    rng = np.random.default_rng(5)
    for d in (4, 12, 64, 100, 128, 200, 256):
        V = 500
        t = rng.standard_normal((V, d)).astype(np.float32)
        bits = (t.view(np.uint32) >> 16).astype(np.uint16)  # a bf16 table (truncated values)
        pr = rng.integers(0, V, size=(3000, 2)).astype(np.int32)
        for dtype, table in ((0, t), (1, bits)):
            ref, bad = oracle_mod.link_scores(table, pr)
            dev = torch.from_numpy(table.view(np.int16) if dtype else table).cuda()
            sc = torch.empty(len(pr), dtype=torch.float32, device="cuda")
            sgns.link_scores(dtype, d, dev, V, torch.from_numpy(pr).cuda(), sc)
            assert np.array_equal(sc.cpu().numpy().view(np.uint32), ref.view(np.uint32)), (d, dtype)
    sc = torch.empty(2, dtype=torch.float32, device="cuda")
    with pytest.raises(sgns.SgnsError) as e:
        sgns.link_scores(0, 4, torch.zeros(10, 4, device="cuda"), 10,
                         torch.tensor([[0, 1], [3, 10]], dtype=torch.int32, device="cuda"), sc)
    assert e.value.status == sgns.EINVAL


@pytest.mark.gpu
def test_device_auc_equals_host_auc(sgns_lib):
    """AUC from GPU scores of the trainer's own table equals the host computation on the
    same embedding (continuous scores: the summation order changes no ranking here)."""
    import synth

    V = 2000
    ip, ix, _ = synth.sbm(V, 8000, blocks=4, ratio=20.0, seed=51)
    tr_ip, tr_ix, pos, neg = synth.holdout(ip, ix, 0.1, seed=52)
    c = synth.random_walks(tr_ip, tr_ix, 5, 40, seed=53).numpy().astype(np.int32)
    counts = np.bincount(c[c >= 0], minlength=V).astype(np.int32)
    with sgns.Trainer(size=64, window=5, negative=5, iter=2, table_size=1000000, debug=0, storage="bf16") as t:
        t.set_vocab(counts)
        t.train_corpus(c)
        a_dev = synth.link_auc_device(t, pos, neg)
        emb = np.zeros((V, 64), np.float32)
        emb[t.order()] = t.embeddings(0)
    a_host = synth.link_auc(emb, pos, neg)
    assert 0.5 < a_dev < 1.0 and abs(a_dev - a_host) < 1e-3
