"""GPU trainers against the reference's golden vectors and the oracle.

With one worker the trainers follow the reference's single-compute-thread order, so
results must be identical bit for bit: the plain engine against the reference policy
(and the reference's own golden outputs), the persistent engine against the oracle's
GPU-resident window policy, in fp32 and in bf16 with stochastic rounding."""
import glob
import hashlib
import json
import os

import numpy as np
import pytest

import sgns
from random_configs import random_case

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# the reference-output cases: a .json (flags, digests) with its .npz (corpus, rows)
GOLDEN_CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def golden(name):
    meta = json.load(open(os.path.join(GOLDEN, name + ".json")))
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return meta, z["corpus"]


def synthetic(name):
    import torch
    import synth

    if name == "cl_d128":
        ip, ix = synth.chung_lu(3000, 20000, 2.1, seed=21)
        c = synth.random_walks(ip, ix, 3, 40, seed=22)
        return dict(V=3000, d=128, window=10, negative=5, iter=1, sample=1e-3, alpha=0.01), c.numpy()
    if name == "cl_d256_k10":
        ip, ix = synth.chung_lu(2000, 12000, 2.1, seed=23)
        L = synth.walk_lengths(2000 * 2, "geometric", mean=30, cap=80, seed=24)
        c = synth.random_walks(ip, ix, 2, L, seed=25)
        return dict(V=2000, d=256, window=5, negative=10, iter=2, sample=1e-3, alpha=0.025), c.numpy()
    if name == "sbm_d64_w15":
        ip, ix, _ = synth.sbm(2400, 12000, seed=26)
        L = synth.walk_lengths(2400 * 2, "uniform", lo=5, hi=120, seed=27)
        c = synth.random_walks(ip, ix, 2, L, seed=28)
        return dict(V=2400, d=64, window=15, negative=3, iter=1, sample=1e-4, alpha=0.02), c.numpy()
    raise KeyError(name)


ALL_CASES = GOLDEN_CASES + ["cl_d128", "cl_d256_k10", "sbm_d64_w15"]


def case(name):
    if name in GOLDEN_CASES:
        meta, corpus = golden(name)
        cfg = {k: meta[k] for k in ("V", "d", "window", "negative", "iter", "sample", "alpha")}
        return cfg, corpus, meta
    cfg, corpus = synthetic(name)
    return cfg, corpus.astype(np.int32), None


def gpu_train(cfg, corpus, engine, storage, workers=1, wpc=1, table_size=None, table_threads=2, mode="hogwild",
              tile=0, windows=2):
    counts = np.bincount(corpus[corpus >= 0], minlength=cfg["V"]).astype(np.int32)
    opt = sgns.default_options(size=cfg["d"], window=cfg["window"], negative=cfg["negative"], iter=cfg["iter"],
                               sample=cfg["sample"], alpha=cfg["alpha"], engine=engine, storage=storage,
                               workers=workers, warps_per_cta=wpc, threads=table_threads,
                               table_size=table_size or 1000000, debug=0, mode=mode, forward_tile=tile,
                               windows_per_step=windows)
    with sgns.Trainer(opt) as t:
        t.set_vocab(counts)
        st = t.train_corpus(corpus)
        return t.embeddings(0), t.embeddings(1), st, t.order()


def oracle_train(oracle_mod, cfg, corpus, policy, storage, workers=1, table_size=None, table_threads=2, windows=2):
    counts = np.bincount(corpus[corpus >= 0], minlength=cfg["V"]).astype(np.int32)
    st = {"fp32": oracle_mod.STORE_F32, "bf16": oracle_mod.STORE_BF16}[storage]
    wih, woh, stats = oracle_mod.train(corpus, counts, d=cfg["d"], window=cfg["window"], negative=cfg["negative"],
                                       iter=cfg["iter"], workers=workers, threads=1, table_threads=table_threads,
                                       policy=policy, storage=st, table_size=table_size or 1000000,
                                       sample=cfg["sample"], alpha=cfg["alpha"], windows=windows)
    if storage == "bf16":
        wih, woh = oracle_mod.bf16_to_f32(wih), oracle_mod.bf16_to_f32(woh)
    return wih, woh, stats


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_plain_fp32_reproduces_reference_outputs(name, sgns_lib):
    cfg, corpus, meta = case(name)
    wih, woh, st, order = gpu_train(cfg, corpus, "plain", "fp32", table_size=meta["table_size"])
    assert np.array_equal(order, np.load(os.path.join(GOLDEN, name + ".npz"))["order"])
    assert sha(wih) == meta["wih_sha256"], np.abs(wih[0] - np.array(meta["wih_row0"], np.float32)).max()
    assert sha(woh) == meta["woh_sha256"]


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_text_output_is_the_references(name, sgns_lib, tmp_path):
    """sgns_save_text after a one-worker plain FP32 run writes the reference's own -eoutput
    file (my_saveModel, dsgl.hpp:1443-1461) byte for byte."""
    meta, corpus = golden(name)
    counts = np.bincount(corpus[corpus >= 0], minlength=meta["V"]).astype(np.int32)
    opt = sgns.default_options(size=meta["d"], window=meta["window"], negative=meta["negative"], iter=meta["iter"],
                               sample=meta["sample"], alpha=meta["alpha"], engine="plain", storage="fp32",
                               mode="exact", threads=2, table_size=meta["table_size"], debug=0)
    out = str(tmp_path / "emb.txt")
    with sgns.Trainer(opt) as t:
        t.set_vocab(counts)
        t.train_corpus(corpus)
        t.save_text(out)
    assert hashlib.sha256(open(out, "rb").read()).hexdigest() == meta["text_sha256"]


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_command_line_trainer_on_walk_files(name, sgns_lib, tmp_path):
    """The sgns_train command line on the golden corpus written as walk files (" %u" per
    vertex, one walk per line; named by a wildcard) reproduces the reference's embedding
    file byte for byte."""
    import subprocess
    import synth

    meta, corpus = golden(name)
    if corpus[0] == -1 or np.any((corpus[:-1] == -1) & (corpus[1:] == -1)):
        pytest.skip("holds an empty walk, which a walk file cannot express")
    # two files split at a walk boundary, named by a wildcard (sorted: walks-0, walks-1)
    ends = np.flatnonzero(corpus == -1)
    cut = int(ends[len(ends) // 2]) + 1
    synth.write_walk_file(corpus[:cut], str(tmp_path / "walks-0.txt"))
    synth.write_walk_file(corpus[cut:], str(tmp_path / "walks-1.txt"))
    walks = str(tmp_path / "walks-*.txt")
    out = str(tmp_path / "emb.txt")
    cli = os.path.join(os.path.dirname(sgns.LIB_PATH), "sgns_train")
    cmd = [cli, "-train", walks, "-eoutput", out, "-size", str(meta["d"]), "-window", str(meta["window"]),
           "-negative", str(meta["negative"]), "-iter", str(meta["iter"]), "-sample", repr(meta["sample"]),
           "-alpha", repr(meta["alpha"]), "-threads", "2", "-debug", "0", "-engine", "plain", "-mode", "exact",
           "-vertices", str(meta["V"]), "-table-size", str(meta["table_size"])]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert hashlib.sha256(open(out, "rb").read()).hexdigest() == meta["text_sha256"]


@pytest.mark.parametrize("storage", ["fp32", "bf16"])
@pytest.mark.parametrize("name", ALL_CASES)
def test_plain_matches_oracle(name, storage, sgns_lib, oracle_mod):
    cfg, corpus, _ = case(name)
    wih, woh, st, _ = gpu_train(cfg, corpus, "plain", storage)
    owih, owoh, ost = oracle_train(oracle_mod, cfg, corpus, oracle_mod.POLICY_REF, storage)
    assert (st.steps, st.pairs, st.word_count_actual) == (ost["steps"], ost["pairs"], ost["word_count_actual"])
    assert np.array_equal(wih.view(np.uint32), owih.view(np.uint32)), np.abs(wih - owih).max()
    assert np.array_equal(woh.view(np.uint32), owoh.view(np.uint32)), np.abs(woh - owoh).max()


@pytest.mark.parametrize("wpc", [1, 2])
@pytest.mark.parametrize("storage", ["fp32", "bf16"])
@pytest.mark.parametrize("name", ALL_CASES)
def test_persistent_matches_oracle(name, storage, wpc, sgns_lib, oracle_mod):
    cfg, corpus, _ = case(name)
    wih, woh, st, _ = gpu_train(cfg, corpus, "persistent", storage, wpc=wpc)
    owih, owoh, ost = oracle_train(oracle_mod, cfg, corpus, oracle_mod.POLICY_WINDOW, storage)
    assert (st.steps, st.pairs, st.word_count_actual) == (ost["steps"], ost["pairs"], ost["word_count_actual"])
    assert abs(st.final_alpha - ost["final_alpha"]) == 0
    assert np.array_equal(wih.view(np.uint32), owih.view(np.uint32)), np.abs(wih - owih).max()
    assert np.array_equal(woh.view(np.uint32), owoh.view(np.uint32)), np.abs(woh - owoh).max()


@pytest.mark.parametrize("engine,storage", [("plain", "fp32"), ("persistent", "fp32"), ("persistent", "bf16")])
@pytest.mark.parametrize("name", ["cl_d128", "basic", "sbm_d64_w15"])
def test_single_window_steps_match_oracle(name, engine, storage, sgns_lib, oracle_mod):
    """windows_per_step = 1: one walk per step, its window and target with the shared
    negatives; bit for bit the oracle's statement of the same step, one worker."""
    cfg, corpus, _ = case(name)
    wih, woh, st, _ = gpu_train(cfg, corpus, engine, storage, windows=1)
    policy = oracle_mod.POLICY_REF if engine == "plain" else oracle_mod.POLICY_WINDOW
    owih, owoh, ost = oracle_train(oracle_mod, cfg, corpus, policy, storage, windows=1)
    assert (st.steps, st.pairs, st.word_count_actual) == (ost["steps"], ost["pairs"], ost["word_count_actual"])
    assert np.array_equal(wih.view(np.uint32), owih.view(np.uint32))
    assert np.array_equal(woh.view(np.uint32), owoh.view(np.uint32))
    # one window per step: about half the pairs of a two-window step
    _, _, st2, _ = gpu_train(cfg, corpus, engine, storage)
    assert st.steps > 1.5 * st2.steps and st.pairs < 0.8 * st2.pairs * st.steps / st2.steps


@pytest.mark.parametrize("tile", [1, 2])
@pytest.mark.parametrize("storage", ["fp32", "bf16"])
@pytest.mark.parametrize("name", ["cl_d128", "basic"])
def test_forward_tiles_match_oracle(name, storage, tile, sgns_lib, oracle_mod):
    """Both forward tiles (one or two lanes per input) compute the window policy's sums in
    the same order: bit for bit the oracle, one worker."""
    cfg, corpus, _ = case(name)
    wih, woh, st, _ = gpu_train(cfg, corpus, "persistent", storage, tile=tile)
    owih, owoh, _ = oracle_train(oracle_mod, cfg, corpus, oracle_mod.POLICY_WINDOW, storage)
    assert st.forward_tile == tile and st.warps_per_worker == 1
    assert np.array_equal(wih.view(np.uint32), owih.view(np.uint32))
    assert np.array_equal(woh.view(np.uint32), owoh.view(np.uint32))


@pytest.mark.parametrize("engine,storage", [("plain", "fp32"), ("persistent", "fp32"), ("persistent", "bf16")])
def test_replay_exact_mode_on_the_10k_vertex_case(engine, storage, sgns_lib, oracle_mod):
    """Replay-exact mode (no worker count given) on a 10,000-vertex Chung-Lu graph
    (98k edges, gamma 2.1), one uniform walk of 80 per vertex (0.8M tokens), d=128, w=10,
    K=5, sample 1e-3, alpha 0.01, unigram table 1e7: one worker, bit for bit the oracle."""
    import synth

    ip, ix = synth.chung_lu(10000, 100000, 2.1, seed=1001)
    corpus = synth.random_walks(ip, ix, 1, 80, seed=1002).numpy().astype(np.int32)
    cfg = dict(V=10000, d=128, window=10, negative=5, iter=1, sample=1e-3, alpha=0.01)
    wih, woh, st, _ = gpu_train(cfg, corpus, engine, storage, workers=0, wpc=0, table_size=10_000_000,
                                mode="exact")
    policy = oracle_mod.POLICY_REF if engine == "plain" else oracle_mod.POLICY_WINDOW
    owih, owoh, ost = oracle_train(oracle_mod, cfg, corpus, policy, storage, table_size=10_000_000)
    assert st.workers == 1
    assert (st.steps, st.pairs, st.word_count_actual) == (ost["steps"], ost["pairs"], ost["word_count_actual"])
    assert np.array_equal(wih.view(np.uint32), owih.view(np.uint32)), np.abs(wih - owih).max()
    assert np.array_equal(woh.view(np.uint32), owoh.view(np.uint32)), np.abs(woh - owoh).max()


@pytest.mark.parametrize("engine", ["plain", "persistent"])
@pytest.mark.parametrize("storage", ["fp32", "bf16"])
def test_loss_accumulation_leaves_training_unchanged(engine, storage, sgns_lib):
    """compute_loss selects a kernel that also sums the SGNS loss; with one worker the
    tables it trains are bit for bit those of the kernel without it."""
    cfg, corpus, _ = case("cl_d128")
    counts = np.bincount(corpus[corpus >= 0], minlength=cfg["V"]).astype(np.int32)
    out = []
    for loss in (0, 1):
        opt = sgns.default_options(size=cfg["d"], window=cfg["window"], negative=cfg["negative"], iter=1,
                                   sample=cfg["sample"], alpha=cfg["alpha"], engine=engine, storage=storage,
                                   workers=1, warps_per_cta=1, table_size=1000000, debug=0, compute_loss=loss)
        with sgns.Trainer(opt) as t:
            t.set_vocab(counts)
            st = t.train_corpus(corpus)
            out.append((t.embeddings(0), t.embeddings(1), st))
    assert np.array_equal(out[0][0].view(np.uint32), out[1][0].view(np.uint32))
    assert np.array_equal(out[0][1].view(np.uint32), out[1][1].view(np.uint32))
    assert out[0][2].loss == 0.0 and np.isfinite(out[1][2].loss) and out[1][2].loss > 0.0
    assert (out[0][2].steps, out[0][2].pairs) == (out[1][2].steps, out[1][2].pairs)


def test_pinned_host_corpus_is_read_in_place(sgns_lib):
    """A corpus in pinned host memory is mapped by the kernel without a staging copy; the
    model equals the one trained from pageable memory, and bad ids are still rejected."""
    import torch

    cfg, corpus, _ = case("cl_d128")
    counts = np.bincount(corpus[corpus >= 0], minlength=cfg["V"]).astype(np.int32)
    pinned = torch.empty(len(corpus) + 3, dtype=torch.int32, pin_memory=True)
    out = []
    for src in ("pageable", "pinned", "pinned+4"):
        opt = sgns.default_options(size=cfg["d"], window=cfg["window"], negative=cfg["negative"], iter=1,
                                   sample=cfg["sample"], alpha=cfg["alpha"], engine="persistent", storage="bf16",
                                   mode="exact", table_size=1000000, debug=0)
        with sgns.Trainer(opt) as t:
            t.set_vocab(counts)
            if src == "pageable":
                st = t.train_corpus(corpus)
            else:
                off = 0 if src == "pinned" else 1  # 4 bytes in: not 16-byte aligned
                pinned[off:off + len(corpus)].copy_(torch.from_numpy(corpus))
                st = t.train_corpus_ptr(pinned.data_ptr() + 4 * off, len(corpus))
            out.append((t.embeddings(0), st.pairs))
    for w, pairs in out[1:]:
        assert pairs == out[0][1] and np.array_equal(w.view(np.uint32), out[0][0].view(np.uint32))
    bad = corpus.copy()
    bad[17] = cfg["V"] + 5
    pinned[:len(bad)].copy_(torch.from_numpy(bad))
    with sgns.Trainer(size=cfg["d"], window=cfg["window"], negative=cfg["negative"], table_size=1000000,
                      debug=0) as t:
        t.set_vocab(counts)
        with pytest.raises(sgns.SgnsError) as e:
            t.train_corpus_ptr(pinned.data_ptr(), len(bad))
        assert e.value.status == sgns.EINVAL


def test_embeddings_into_pinned_host_memory(sgns_lib):
    """BF16 tables read into pinned host memory (16-byte aligned: written in place by the
    widening kernel; 4 bytes in: through the staging buffer) equal the read into pageable
    memory, bit for bit."""
    import torch

    cfg, corpus, _ = case("cl_d128")
    counts = np.bincount(corpus[corpus >= 0], minlength=cfg["V"]).astype(np.int32)
    opt = sgns.default_options(size=cfg["d"], window=cfg["window"], negative=cfg["negative"], iter=1,
                               sample=cfg["sample"], alpha=cfg["alpha"], engine="persistent", storage="bf16",
                               table_size=1000000, debug=0)
    with sgns.Trainer(opt) as t:
        t.set_vocab(counts)
        t.train_corpus(corpus)
        for which in (0, 1):
            want = t.embeddings(which)
            pinned = torch.full((want.size + 4,), float("nan"), dtype=torch.float32, pin_memory=True)
            for off in (0, 1):
                t.embeddings_to(which, pinned.data_ptr() + 4 * off)
                got = pinned[off:off + want.size].numpy().reshape(want.shape)
                assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (which, off)


@pytest.mark.parametrize("seed", [101, 303, 1002, 1003, 2054, 2192])
@pytest.mark.parametrize("engine,storage", [("plain", "fp32"), ("persistent", "fp32"), ("persistent", "bf16")])
def test_engines_match_oracle_on_random_configs(seed, engine, storage, sgns_lib, oracle_mod):
    cfg, corpus = random_case(seed)
    wih, woh, st, _ = gpu_train(cfg, corpus, engine, storage, workers=0, wpc=0, mode="exact")
    policy = oracle_mod.POLICY_REF if engine == "plain" else oracle_mod.POLICY_WINDOW
    owih, owoh, ost = oracle_train(oracle_mod, cfg, corpus, policy, storage)
    assert (st.steps, st.pairs, st.word_count_actual) == (ost["steps"], ost["pairs"], ost["word_count_actual"]), cfg
    assert np.array_equal(wih.view(np.uint32), owih.view(np.uint32)), (cfg, np.abs(wih - owih).max())
    assert np.array_equal(woh.view(np.uint32), owoh.view(np.uint32)), (cfg, np.abs(woh - owoh).max())


def test_autotuner_cache_file(sgns_lib, tmp_path, monkeypatch):
    """With SGNS_TUNE_CACHE set, the autotuner records its choice per device and shape and a
    later run takes the recorded shape instead of tuning again."""
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("SGNS_TUNE_CACHE", str(cache))
    cfg, corpus, _ = case("cl_d128")
    counts = np.bincount(corpus[corpus >= 0], minlength=cfg["V"]).astype(np.int32)

    def run():
        with sgns.Trainer(size=cfg["d"], window=cfg["window"], negative=cfg["negative"], table_size=1000000,
                          debug=0, storage="bf16") as t:
            t.set_vocab(counts)
            st = t.train_corpus(corpus)
            return st.warps_per_cta, st.forward_tile

    first, tile = run()
    lines = cache.read_text().splitlines()
    assert len(lines) == 1 and lines[0].endswith("\t%d\t%d" % (first, tile)) and tile in (1, 2)
    planted = 3 if first != 3 else 2  # the last entry of a key wins
    cache.write_text(lines[0].split("\t")[0] + "\t%d\t%d\n" % (planted, 3 - tile), encoding="utf-8")
    assert run() == (planted, 3 - tile)


@pytest.mark.parametrize("engine,policy", [("plain", 0), ("persistent", 1)])
def test_many_workers_follow_the_reference_control_flow(engine, policy, sgns_lib, oracle_mod):
    """Hogwild workers race on table rows, but every worker's control flow (slice,
    subsampling, windows, negatives, learning-rate schedule inputs) is independent of
    the table values: step, pair and word counts equal the oracle's exactly."""
    cfg, corpus, _ = case("cl_d128")
    W = 37
    wih, woh, st, _ = gpu_train(cfg, corpus, engine, "fp32", workers=W, wpc=1)
    owih, owoh, ost = oracle_train(oracle_mod, cfg, corpus, policy, "fp32", workers=W)
    assert (st.steps, st.pairs, st.word_count_actual) == (ost["steps"], ost["pairs"], ost["word_count_actual"])
    assert np.isfinite(wih).all() and np.isfinite(woh).all()


def test_invalid_vertex_id_is_rejected(sgns_lib):
    opt = sgns.default_options(size=8, window=2, negative=2, iter=1, debug=0, table_size=1000)
    with sgns.Trainer(opt) as t:
        t.set_vocab(np.ones(10, np.int32))
        with pytest.raises(sgns.SgnsError) as e:
            t.upload(np.array([1, 2, 10, -1], np.int32))
        assert e.value.status == sgns.EINVAL
        with pytest.raises(sgns.SgnsError):
            t.upload(np.array([1, -2, 3, -1], np.int32))


def test_empty_and_degenerate_corpora(sgns_lib):
    opt = sgns.default_options(size=8, window=2, negative=2, iter=2, debug=0, table_size=1000)
    for eng in ("plain", "persistent"):
        opt.engine = {"plain": 0, "persistent": 1}[eng]
        with sgns.Trainer(opt) as t:
            t.set_vocab(np.ones(10, np.int32))
            w0 = t.embeddings(0)
            st = t.train_corpus(np.array([], np.int32))
            assert st.steps == 0
            st = t.train_corpus(np.array([-1, -1, 3, -1, 4, -1], np.int32))  # only length-1 walks
            assert st.steps == 0
            assert np.array_equal(t.embeddings(0), w0)


def _hold_all_but(nbytes):
    """Device memory held by torch so that about nbytes stay free."""
    import torch

    free, _ = torch.cuda.mem_get_info()
    return torch.empty(max(0, free - nbytes), dtype=torch.uint8, device="cuda")


def test_failed_vocabulary_leaves_the_handle_without_one(sgns_lib):
    """Tables that do not fit: sgns_set_vocab fails with ENOMEM and leaves the handle as
    before any vocabulary (training refused with ESTATE, nothing half-allocated); a
    vocabulary that fits then trains."""
    import torch

    opt = sgns.default_options(size=256, window=2, negative=2, iter=1, debug=0, table_size=1000, sample=0.0,
                               workers=1, warps_per_cta=1)
    with sgns.Trainer(opt) as t:
        hold = _hold_all_but(3 << 29)  # 1.5 GiB free; the two tables need 2 GiB
        try:
            with pytest.raises(sgns.SgnsError) as e:
                t.set_vocab(np.ones(1 << 20, np.int32))
            assert e.value.status == sgns.ENOMEM
        finally:
            del hold
            torch.cuda.empty_cache()
        assert t.vocab_size == 0
        with pytest.raises(sgns.SgnsError) as e:
            t.train()
        assert e.value.status == sgns.ESTATE
        t.set_vocab(np.ones(10, np.int32))
        walks = np.random.default_rng(3).integers(0, 10, (30, 6))
        st = t.train_corpus(np.hstack([walks, -np.ones((30, 1), np.int64)]).ravel().astype(np.int32))
        assert st.steps > 0 and np.isfinite(t.embeddings(0)).all()


def test_autotuner_without_room_for_scratch_tables(sgns_lib):
    """When the autotuner's scratch copies of the tables do not fit, the engine runs at the
    most warps per CTA that fit instead of failing, and trains the same control flow."""
    import torch

    rng = np.random.default_rng(7)
    V = 1 << 20
    corpus = np.concatenate([np.append(rng.integers(0, V, 60), -1) for _ in range(4000)]).astype(np.int32)
    counts = np.bincount(corpus[corpus >= 0], minlength=V).astype(np.int32)
    counts[counts == 0] = 1
    opt = sgns.default_options(size=256, window=5, negative=5, iter=1, debug=0, table_size=1000000)
    with sgns.Trainer(opt) as t:
        t.set_vocab(counts)  # two 1 GiB tables
        t.upload(corpus)
        hold = _hold_all_but(3 << 29)  # room for one scratch table, not two
        try:
            st = t.train()
        finally:
            del hold
            torch.cuda.empty_cache()
        assert 1 <= st.warps_per_cta <= 8 and st.steps > 0 and st.pairs > 0
        assert np.isfinite(t.embeddings(0)).all() and np.isfinite(t.embeddings(1)).all()
