"""Link-prediction AUC of the CPU trainer on fixed SBM corpora -- the fixture that the GPU
engines' AUC is compared with (bench.py's auc_sbm leg).

Configuration 2: a 4-block stochastic block model (p_in / p_out = 20, about
2.73 undirected edges per vertex), 10% of the edges held out as in src/tools/gtrain.cpp
:293-333, 10 information-oriented walks per vertex (the entropy/length stop rule of
include/walk.hpp:260-387, 868-874, min length 20, capped at 80 vertices, R threshold 0.84
for a mean length near 40), d = 128, window 10, 5 negatives, sample 1e-3, alpha 0.01, one
pass, unigram table 1e8.

The walks make no trace steps (sgns_walk_options.trace_steps = 0).  On this graph nearly
no edge has a common neighbour, so the reference's trace step returns to the current
vertex on about 80% of the moves; walks then cover only a few hops and the one-pass
training links held-out edges barely better than chance (AUC 0.54 for the CPU trainer and
for the reference's own trainer on one seed, recorded under "trace_walks"), which cannot
tell engines apart.  Without trace steps the same stop rule gives AUC near 0.78.

Everything is drawn on the CPU from fixed seeds with platform-independent integer
arithmetic (synth.sbm_csr, synth.holdout_csr, the oracle's walker), so the GPU side can
rebuild the identical corpus and check it against the SHA-256 recorded here.  The CPU
trainer is the oracle's restatement of include/dsgl.hpp with the reference's buffer
policy and Hogwild threads; for one seed the reference's own trainer (compiled here by
oracle/build_ref.sh) is recorded beside it.  Test infrastructure: run from the
repository root (the reference run needs the reference checkout's build):
    python tests/golden/make_auc_fixture.py [--vertices 100000 1100000] [--seeds 1 2 3]
"""
import argparse
import hashlib
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
for _p in (os.path.join(ROOT, "gdistger-re_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)
OUT = os.path.join(ROOT, "tests", "golden", "auc_sbm.json")
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "dsgl_ref")

GRAPH = dict(edges_per_vertex=2.73, blocks=4, ratio=20.0, holdout=0.1)
WALKS = dict(walks_per_vertex=10, min_length=20, max_length=80, r_threshold=0.84, trace_steps=0)
# the reference's trace steps on the same graph (one recorded case; see above)
TRACE_WALKS = dict(walks_per_vertex=10, min_length=20, max_length=80, r_threshold=0.78, trace_steps=1)
TRAIN = dict(size=128, window=10, negative=5, sample=1e-3, alpha=0.01, iter=1, table_size=100_000_000,
             table_threads=12)


def seeds_of(seed):
    """Graph, holdout and walk seeds of one case."""
    return dict(graph=seed, holdout=1000 + seed, walks=2000 + seed)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def build_case(V, seed, walks=WALKS):
    """(train_indptr, train_indices, pos, neg, corpus, info) of one case, on the CPU."""
    import oracle
    import synth

    s = seeds_of(seed)
    ip, ix, _ = synth.sbm_csr(V, int(GRAPH["edges_per_vertex"] * V), GRAPH["blocks"], GRAPH["ratio"], seed=s["graph"])
    tip, tix, pos, neg = synth.holdout_csr(ip, ix, GRAPH["holdout"], seed=s["holdout"])
    cn = oracle.edge_common_neighbors(tip, tix)
    corpus, lengths = oracle.info_walks(tip, tix, cn, walks["walks_per_vertex"] * V, walks["min_length"],
                                        walks["max_length"], walks["r_threshold"], s["walks"], walks["trace_steps"])
    info = dict(V=V, seed=seed, seeds=s, edges=int(len(ix) // 2), train_edges=int(len(tix) // 2),
                holdout=int(pos.shape[1]), tokens=int(len(corpus)), walk_mean_length=float(lengths.mean()),
                graph_sha256=sha(np.concatenate([tip.view(np.int32), tix])), pos_sha256=sha(pos),
                neg_sha256=sha(neg), corpus_sha256=sha(corpus))
    return tip, tix, pos, neg, corpus, info


def embedding_auc(wih_sorted, order, V, pos, neg):
    import synth

    emb = np.zeros((V, wih_sorted.shape[1]), np.float32)
    emb[order] = wih_sorted
    return synth.link_auc(emb, pos, neg)


def cpu_trainer(corpus, V, pos, neg, threads):
    import oracle

    counts = np.bincount(corpus[corpus >= 0], minlength=V).astype(np.int32)
    t0 = time.time()
    wih, _, st = oracle.train(corpus, counts, d=TRAIN["size"], window=TRAIN["window"], negative=TRAIN["negative"],
                              iter=TRAIN["iter"], workers=threads, threads=threads,
                              table_threads=TRAIN["table_threads"], policy=oracle.POLICY_REF,
                              storage=oracle.STORE_F32, table_size=TRAIN["table_size"], sample=TRAIN["sample"],
                              alpha=TRAIN["alpha"])
    order, _, _, _ = oracle.vocab(counts)
    return dict(auc=embedding_auc(wih, order, V, pos, neg), threads=threads, pairs=int(st["pairs"]),
                train_seconds=float(st["train_seconds"]), wall_seconds=time.time() - t0,
                kind="oracle restatement of include/dsgl.hpp, reference buffer policy, fp32, Hogwild threads")


def reference_trainer(corpus, V, pos, neg, threads):
    """The reference's own dsgl() (oracle/_ref/dsgl_ref), threads compute threads."""
    with tempfile.TemporaryDirectory() as tmp:
        cpath = os.path.join(tmp, "corpus.i32")
        corpus.astype(np.int32).tofile(cpath)
        pre = os.path.join(tmp, "out")
        flags = ["-size", str(TRAIN["size"]), "-window", str(TRAIN["window"]), "-negative", str(TRAIN["negative"]),
                 "-sample", str(TRAIN["sample"]), "-alpha", str(TRAIN["alpha"]), "-iter", str(TRAIN["iter"]),
                 "-threads", str(threads + 1), "-min-count", "0", "-batch-size", "21", "-debug", "0",
                 "-eoutput", os.path.join(tmp, "emb.txt")]
        t0 = time.time()
        subprocess.run([REF_BIN, cpath, str(V), pre] + flags, check=True, stdout=subprocess.DEVNULL)
        wall = time.time() - t0
        wih = np.fromfile(pre + ".wih", np.float32).reshape(V, TRAIN["size"])
        order = np.fromfile(pre + ".order", np.uint32)
    return dict(auc=embedding_auc(wih, order, V, pos, neg), threads=threads, wall_seconds=wall,
                kind="the reference's include/dsgl.hpp compiled unmodified (oracle/build_ref.sh), "
                     "compute threads as stated, sequential-k cblas stand-in")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--vertices", type=int, nargs="+", default=[100_000, 1_100_000])
    ap.add_argument("--seeds", type=int, nargs="+", default=[1, 2, 3])
    ap.add_argument("--threads", type=int, default=8)
    ap.add_argument("--reference-seed", type=int, default=1)
    ap.add_argument("--reference-vertices", type=int, nargs="*", default=[100_000])
    ap.add_argument("--trace-case", action="store_true", help="also record the trace-step walks at 100k, seed 1")
    args = ap.parse_args()
    data = json.load(open(OUT)) if os.path.exists(OUT) else {}
    data.update(graph=GRAPH, walks=WALKS, train=TRAIN, generator=os.path.relpath(__file__, ROOT))
    if "trace_walks" not in data and args.trace_case:
        tip, tix, pos, neg, corpus, info = build_case(100_000, 1, TRACE_WALKS)
        info["walks"] = TRACE_WALKS
        info["cpu_trainer"] = cpu_trainer(corpus, 100_000, pos, neg, args.threads)
        if os.path.exists(REF_BIN):
            info["reference"] = reference_trainer(corpus, 100_000, pos, neg, args.threads)
        data["trace_walks"] = info
        with open(OUT, "w") as f:
            json.dump(data, f, indent=1)
    cases = {(c["V"], c["seed"]): c for c in data.get("cases", [])}
    for V in args.vertices:
        for seed in args.seeds:
            tip, tix, pos, neg, corpus, info = build_case(V, seed)
            old = cases.get((V, seed), {})
            if old.get("corpus_sha256") == info["corpus_sha256"] and "cpu_trainer" in old:
                info["cpu_trainer"] = old["cpu_trainer"]
            else:
                info["cpu_trainer"] = cpu_trainer(corpus, V, pos, neg, args.threads)
            if V in args.reference_vertices and seed == args.reference_seed and os.path.exists(REF_BIN):
                if old.get("corpus_sha256") == info["corpus_sha256"] and "reference" in old:
                    info["reference"] = old["reference"]
                else:
                    info["reference"] = reference_trainer(corpus, V, pos, neg, args.threads)
            elif "reference" in old and old.get("corpus_sha256") == info["corpus_sha256"]:
                info["reference"] = old["reference"]
            cases[(V, seed)] = info
            print(json.dumps(info), flush=True)
            data["cases"] = [cases[k] for k in sorted(cases)]
            with open(OUT, "w") as f:
                json.dump(data, f, indent=1)
    summary = {}
    for V in sorted({k[0] for k in cases}):
        a = [cases[k]["cpu_trainer"]["auc"] for k in sorted(cases) if k[0] == V]
        summary[str(V)] = dict(cpu_trainer_auc_mean=float(np.mean(a)), cpu_trainer_auc_std=float(np.std(a)),
                               seeds=len(a))
    data["summary"] = summary
    with open(OUT, "w") as f:
        json.dump(data, f, indent=1)
    print(json.dumps(summary))


if __name__ == "__main__":
    main()
