"""Generates the golden vectors of tests/golden/ by running the reference's own DSGL
trainer (include/dsgl.hpp of trsenli/GDistGER-re, compiled unmodified by
oracle/build_ref.sh against single-rank MPI / cblas stand-ins) on small seeded corpora.

Each case stores the corpus, the flags, the reference's vocabulary order, the SHA-256
of its final Wih and Woh (float32, sorted-row order) and a few rows for diagnosis.
One compute thread (-threads 2: one sync thread + one compute thread) makes the
reference deterministic.  Needs the reference checkout; run from the repository root:
    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
OUT = os.path.join(ROOT, "tests", "golden")
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "dsgl_ref")
TMP = os.path.join(ROOT, "oracle", "_ref", "tmp")


def powerlaw_walks(V, n_walks, lmin, lmax, seed, extra=()):
    rng = np.random.default_rng(seed)
    w = (np.arange(V) + 10.0) ** -0.9
    w /= w.sum()
    toks = []
    for _ in range(n_walks):
        L = int(rng.integers(lmin, lmax + 1))
        toks.extend(rng.choice(V, size=L, p=w).tolist())
        toks.append(-1)
    for walk in extra:
        toks.extend(list(walk))
        toks.append(-1)
    return np.array(toks, dtype=np.int32)


CASES = [
    dict(name="basic", V=1200, d=16, window=5, negative=5, iter=2, sample=1e-3, alpha=0.025,
         walks=dict(n_walks=400, lmin=2, lmax=60, seed=11)),
    dict(name="d128_w10", V=1100, d=128, window=10, negative=5, iter=1, sample=1e-3, alpha=0.01,
         walks=dict(n_walks=150, lmin=40, lmax=80, seed=12)),
    dict(name="edges_nosample", V=1050, d=8, window=3, negative=10, iter=3, sample=0.0, alpha=0.05,
         walks=dict(n_walks=120, lmin=1, lmax=30, seed=13), long_walk=2500),
    dict(name="subsample_k2", V=1500, d=12, window=7, negative=2, iter=1, sample=1e-2, alpha=0.025,
         walks=dict(n_walks=500, lmin=2, lmax=40, seed=14)),
    dict(name="k0_w1", V=1010, d=4, window=1, negative=0, iter=2, sample=1e-3, alpha=0.025,
         walks=dict(n_walks=300, lmin=2, lmax=20, seed=15)),
]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run_case(c):
    extra = []
    if c.get("long_walk"):
        rng = np.random.default_rng(99)
        extra.append(rng.integers(0, c["V"], size=c["long_walk"]).tolist())
        extra.append([])  # an empty walk: two separators in a row
        extra.append([5])  # a walk of length one
    corpus = powerlaw_walks(c["V"], extra=extra, **c["walks"])
    os.makedirs(TMP, exist_ok=True)
    cpath = os.path.join(TMP, c["name"] + ".i32")
    corpus.tofile(cpath)
    pre = os.path.join(TMP, c["name"])
    flags = ["-size", str(c["d"]), "-window", str(c["window"]), "-negative", str(c["negative"]),
             "-iter", str(c["iter"]), "-sample", repr(c["sample"]), "-alpha", repr(c["alpha"]),
             "-threads", "2", "-debug", "0", "-eoutput", pre + ".txt"]
    env = dict(os.environ, DSGL_REF_DUMP_TABLES="1")
    r = subprocess.run([REF_BIN, cpath, str(c["V"]), pre] + flags, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError("reference run failed: %s\n%s" % (r.stdout[-2000:], r.stderr[-2000:]))
    V, d = c["V"], c["d"]
    wih = np.fromfile(pre + ".wih", dtype=np.float32).reshape(V, d)
    woh = np.fromfile(pre + ".woh", dtype=np.float32).reshape(V, d)
    order = np.fromfile(pre + ".order", dtype=np.uint32)
    exp = np.fromfile(pre + ".exp", dtype=np.float32)
    table = np.fromfile(pre + ".table", dtype=np.int32)
    meta = dict(c)
    meta.update(wih_sha256=sha(wih), woh_sha256=sha(woh), table_sha256=sha(table), table_size=int(table.size),
                table_threads=2, exp_sha256=sha(exp), wih_row0=wih[0].tolist(), woh_row0=woh[0].tolist(),
                wih_last=wih[-1].tolist(),
                # the reference's own -eoutput file (my_saveModel, dsgl.hpp:1443-1461)
                text_sha256=hashlib.sha256(open(pre + ".txt", "rb").read()).hexdigest())
    np.savez_compressed(os.path.join(OUT, c["name"] + ".npz"), corpus=corpus, order=order)
    with open(os.path.join(OUT, c["name"] + ".json"), "w") as f:
        json.dump(meta, f, indent=1)
    for ext in (".wih", ".woh", ".order", ".exp", ".table", ".txt", ".i32"):
        try:
            os.remove(pre + ext)
        except FileNotFoundError:
            pass
    return meta


def main():
    subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    names = sys.argv[1:]
    for c in CASES:
        if names and c["name"] not in names:
            continue
        m = run_case(c)
        print(c["name"], m["wih_sha256"][:16], m["woh_sha256"][:16])


if __name__ == "__main__":
    main()
