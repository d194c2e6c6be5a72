"""Information-oriented walks (sgns_info_walks) and per-edge common-neighbour counts
(sgns_edge_common_neighbors): the corpus producer in front of the trainer (include/walk.hpp
:260-387, :818-1042 of the reference), against the oracle's restatement with the same
counter-based random stream (oracle/walk_oracle.cpp), bit for bit."""
import math

import numpy as np
import pytest

import sgns
import synth


def small_graphs():
    """(name, indptr, indices): an SBM, a power-law graph with hubs, and hand-made edge cases
    (isolated vertices, a vertex whose only neighbour is itself, a degree-2 vertex with a
    self loop, a path)."""
    out = []
    ip, ix, _ = synth.sbm_csr(3000, 9000, blocks=4, ratio=20.0, seed=5)
    out.append(("sbm", ip, ix))
    import torch

    cip, cix = synth.chung_lu(2000, 12000, 2.1, seed=6)
    out.append(("chung_lu", cip.numpy().astype(np.int64), cix.numpy().astype(np.int32)))
    # 0: isolated; 1: only itself; 2: {2, 3} (degree 2, self loop first); 3: {2, 4};
    # 4: {3, 5}; 5: {4, 6}; 6: {5}; 7: isolated
    adj = {0: [], 1: [1], 2: [2, 3], 3: [2, 4], 4: [3, 5], 5: [4, 6], 6: [5], 7: []}
    V = len(adj)
    ind = np.array([v for u in range(V) for v in adj[u]], np.int32)
    ipp = np.zeros(V + 1, np.int64)
    ipp[1:] = np.cumsum([len(adj[u]) for u in range(V)])
    out.append(("edge_cases", ipp, ind))
    return out


def python_common_neighbors(ip, ix):
    V = len(ip) - 1
    nb = [set(ix[ip[u]:ip[u + 1]].tolist()) for u in range(V)]
    return np.array([len(nb[u] & nb[int(ix[e])]) for u in range(V) for e in range(ip[u], ip[u + 1])], np.int32)


def python_walk(ip, ix, cn, xl, tanh_pos, w, min_length, max_length, r_th, seed, trace=1):
    """The walker rule as a plain loop (the oracle's arithmetic primitives, small graphs)."""
    M = (1 << 64) - 1
    G = 0x9E3779B97F4A7C15

    def mix(z):
        z = (z + G) & M
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        return z ^ (z >> 31)

    V = len(ip) - 1
    ctr = mix(seed ^ ((w * G) & M))

    def draw():
        nonlocal ctr
        r = mix(ctr)
        ctr = (ctr + G) & M
        return r

    path = [w % V]
    st = dict(H=0.0, EH=0.0, ES=1.0, EHS=0.0, EHH=0.0, ESS=1.0, N=1.0, R=1.0)
    if len(path) >= max_length:
        return path

    def append(v):
        S = len(path)
        f = path.count(v)
        t = ((xl[S] - xl[S + 1]) + xl[f + 1]) - xl[f]
        S1 = float(S + 1)
        H1 = (float(S) * st["H"] - t) / S1
        N1 = st["N"] + 1.0
        st["EH"] += (H1 - st["EH"]) / N1
        st["ES"] += (S1 - st["ES"]) / N1
        st["EHS"] += (H1 * S1 - st["EHS"]) / N1
        st["EHH"] += (H1 * H1 - st["EHH"]) / N1
        st["ESS"] += (S1 * S1 - st["ESS"]) / N1
        DH = st["EHH"] - st["EH"] * st["EH"]
        DS = st["ESS"] - st["ES"] * st["ES"]
        ex = st["EHS"] - st["EH"] * st["ES"]
        q = DH * DS  # C semantics: sqrt of a negative is NaN, x / 0 is +-inf
        if ex == 0.0:
            st["R"] = 0.0
        elif q > 0:
            st["R"] = ex / math.sqrt(q)
        elif q == 0:
            st["R"] = math.copysign(math.inf, ex)
        else:
            st["R"] = float("nan")
        st["H"], st["N"] = H1, N1
        path.append(v)
        moves = len(path) - 1
        R = st["R"]
        if moves > min_length and (R * R < r_th or R < 0.0):
            return True
        return len(path) >= max_length

    cur, redraws = w % V, 0
    while True:
        b, ds = int(ip[cur]), int(ip[cur + 1] - ip[cur])
        if ds == 0:
            break
        e = b + (((draw() >> 32) * ds) >> 32)
        u = int(ix[e])
        if ds == 2 and int(ix[b]) == cur:
            break
        if len(path) == 1 and u == cur:
            redraws += 1
            if redraws >= 64:
                break
            continue
        tr = False
        if trace:
            p = float(draw() >> 11) * (1.0 / 9007199254740992.0)
            du = int(ip[u + 1] - ip[u])
            pa = ((1.0 / float(ds - int(cn[e]))) * float(max(ds, du))) / float(min(ds, du)) if ds > cn[e] else math.inf
            tr = tanh_pos(pa) <= p
        if append(u):
            break
        if tr:
            if append(cur):
                break
        else:
            cur = u
    return path


def test_entropy_table_and_tanh_are_accurate(oracle_mod):
    xl = oracle_mod.xlog2x_table(1002)
    ref = np.array([0.0] + [x * math.log2(x) for x in range(1, 1002)])
    assert np.max(np.abs(xl[1:] - ref[1:]) / ref[1:].clip(min=1e-300)) < 1e-15
    assert xl[0] == 0.0 and xl[1] == 0.0 and xl[2] == 2.0 and xl[1024 // 2] == 512 * 9.0
    for x in np.concatenate([np.linspace(0, 20, 2001), [1e-9, 0.3333, 19.99, 20.0, 1e3, math.inf]]):
        assert abs(oracle_mod.tanh_pos(x) - math.tanh(x)) <= 4e-16 * max(1.0, math.tanh(x)), x


def test_library_entropy_table_equals_oracle(sgns_lib, oracle_mod):
    """The table sgns_info_walks uploads is built on the host by the library: the same bits
    as the oracle's."""
    a, b = sgns.xlog2x_table(1002), oracle_mod.xlog2x_table(1002)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_oracle_common_neighbors_are_set_intersections(oracle_mod):
    for name, ip, ix in small_graphs():
        assert np.array_equal(oracle_mod.edge_common_neighbors(ip, ix), python_common_neighbors(ip, ix)), name


@pytest.mark.parametrize("min_length,max_length,r_th,seed,trace", [(20, 80, 0.999, 1, 1), (20, 80, 0.8, 2, 1),
                                                                   (0, 30, 0.95, 3, 1), (5, 1, 0.9, 4, 1),
                                                                   (3, 1000, 0.5, 5, 1), (20, 80, 0.84, 6, 0)])
def test_oracle_walks_follow_the_rule(oracle_mod, min_length, max_length, r_th, seed, trace):
    """The restated walker against the rule written as a plain loop, walk by walk."""
    xl = oracle_mod.xlog2x_table(1002)
    for name, ip, ix in small_graphs():
        cn = oracle_mod.edge_common_neighbors(ip, ix)
        V = len(ip) - 1
        n = min(3 * V, 600)
        corpus, lengths = oracle_mod.info_walks(ip, ix, cn, n, min_length, max_length, r_th, seed, trace)
        ends = np.flatnonzero(corpus == -1)
        assert len(ends) == n and np.array_equal(np.diff(np.concatenate([[-1], ends])) - 1, lengths)
        starts = np.concatenate([[0], ends[:-1] + 1])
        for w in range(0, n, 7 if V > 100 else 1):
            walk = corpus[starts[w]:ends[w]].tolist()
            ref = python_walk(ip, ix, cn, xl, oracle_mod.tanh_pos, w, min_length, max_length, r_th, seed, trace)
            assert walk == ref, (name, w)


def test_oracle_walk_shapes(oracle_mod):
    """Structure of every walk: it starts at w % V, each step follows an edge or returns to
    the vertex it came from, lengths respect min/max; edge cases end where the rule says."""
    for name, ip, ix in small_graphs():
        cn = oracle_mod.edge_common_neighbors(ip, ix)
        V = len(ip) - 1
        nb = [set(ix[ip[u]:ip[u + 1]].tolist()) for u in range(V)]
        corpus, lengths = oracle_mod.info_walks(ip, ix, cn, 2 * V, 4, 60, 0.9, 9)
        ends = np.flatnonzero(corpus == -1)
        starts = np.concatenate([[0], ends[:-1] + 1])
        for w in range(2 * V):
            walk = corpus[starts[w]:ends[w]]
            assert walk[0] == w % V and 1 <= len(walk) <= 60
            for a, b in zip(walk[:-1], walk[1:]):
                assert b in nb[a], (name, w)
            if ip[walk[0] + 1] > ip[walk[0]] and len(walk) < 60 and name != "edge_cases":
                assert len(walk) >= 4 + 1
        if name == "edge_cases":
            L = lengths[:V].tolist()
            assert L[0] == 1 and L[7] == 1  # isolated vertices
            assert L[1] == 1                # only itself: 64 redraws, then the walk ends
            assert L[2] == 1                # degree 2 with the self loop first ends at once


@pytest.mark.gpu
def test_gpu_common_neighbors_match_oracle(sgns_lib, oracle_mod):
    import torch

    for name, ip, ix in small_graphs():
        ref = oracle_mod.edge_common_neighbors(ip, ix)
        cn = torch.full((len(ix),), -7, dtype=torch.int32, device="cuda")
        sgns.edge_common_neighbors(torch.from_numpy(ip).cuda(), torch.from_numpy(ix).cuda(), cn)
        assert np.array_equal(cn.cpu().numpy(), ref), name


@pytest.mark.gpu
@pytest.mark.parametrize("min_length,max_length,r_th,seed,trace", [(20, 80, 0.999, 1, 1), (20, 80, 0.78, 2, 1),
                                                                   (0, 30, 0.95, 3, 1), (5, 1, 0.9, 4, 1),
                                                                   (3, 1000, 0.5, 5, 1), (20, 200, 0.7, 6, 1),
                                                                   (20, 80, 0.84, 7, 0), (0, 1000, 0.6, 8, 0)])
def test_gpu_walks_match_oracle(sgns_lib, oracle_mod, min_length, max_length, r_th, seed, trace):
    import torch

    for name, ip, ix in small_graphs():
        cn = oracle_mod.edge_common_neighbors(ip, ix)
        n = 5 * (len(ip) - 1) + 3
        ref, _ = oracle_mod.info_walks(ip, ix, cn, n, min_length, max_length, r_th, seed, trace)
        dip, dix, dcn = (torch.from_numpy(a).cuda() for a in (ip, ix, cn))
        out, n_tok = sgns.info_walks(dip, dix, dcn, n, min_length, max_length, r_th, seed, trace=trace)
        assert n_tok == len(ref) and np.array_equal(out.cpu().numpy(), ref), (name, n_tok, len(ref))


@pytest.mark.gpu
def test_gpu_walks_at_scale_match_oracle(sgns_lib, oracle_mod):
    """A 200k-vertex SBM, 2 walkers per vertex, the configuration's rule (min 20, cap 80)."""
    import torch

    ip, ix, _ = synth.sbm_csr(200_000, 546_000, blocks=4, ratio=20.0, seed=8)
    tip, tix, _, _ = synth.holdout_csr(ip, ix, 0.1, seed=9)
    cn = oracle_mod.edge_common_neighbors(tip, tix)
    dip, dix = torch.from_numpy(tip).cuda(), torch.from_numpy(tix).cuda()
    dcn = torch.empty(len(tix), dtype=torch.int32, device="cuda")
    sgns.edge_common_neighbors(dip, dix, dcn)
    assert np.array_equal(dcn.cpu().numpy(), cn)
    for trace, r_th in ((1, 0.78), (0, 0.84)):
        ref, _ = oracle_mod.info_walks(tip, tix, cn, 400_000, 20, 80, r_th, 10, trace)
        out, n_tok = sgns.info_walks(dip, dix, dcn, 400_000, 20, 80, r_th, 10, trace=trace)
        assert n_tok == len(ref) and np.array_equal(out.cpu().numpy(), ref), trace


@pytest.mark.gpu
def test_gpu_walk_arguments_are_checked(sgns_lib):
    import torch

    ip = torch.tensor([0, 1, 2], dtype=torch.int64, device="cuda")
    ix = torch.tensor([1, 0], dtype=torch.int32, device="cuda")
    cn = torch.zeros(2, dtype=torch.int32, device="cuda")
    out, n = sgns.info_walks(ip, ix, cn, 4, 0, 5, 0.9, 1)
    assert n == len(out) and (out.cpu().numpy() == -1).sum() == 4
    small = torch.empty(2, dtype=torch.int32, device="cuda")
    with pytest.raises(sgns.SgnsError) as e:  # capacity too small: EINVAL, count reported
        sgns.info_walks(ip, ix, cn, 4, 0, 5, 0.9, 1, corpus=small)
    assert e.value.status == sgns.EINVAL
    bad_cases = [
        (torch.tensor([0, 1, 3], dtype=torch.int64, device="cuda"), ix),      # indptr[V] != E
        (torch.tensor([0, 2, 1], dtype=torch.int64, device="cuda"), ix),      # decreasing
        (ip, torch.tensor([1, 2], dtype=torch.int32, device="cuda")),         # id outside [0, V)
    ]
    for bip, bix in bad_cases:
        with pytest.raises(sgns.SgnsError) as e:
            sgns.info_walks(bip, bix, cn, 4, 0, 5, 0.9, 1)
        assert e.value.status == sgns.EINVAL
        with pytest.raises(sgns.SgnsError) as e:
            sgns.edge_common_neighbors(bip, bix, cn)
        assert e.value.status == sgns.EINVAL
    with pytest.raises(sgns.SgnsError) as e:  # adjacency not strictly increasing
        sgns.edge_common_neighbors(torch.tensor([0, 2, 3, 4], dtype=torch.int64, device="cuda"),
                                   torch.tensor([2, 1, 0, 0], dtype=torch.int32, device="cuda"),
                                   torch.zeros(4, dtype=torch.int32, device="cuda"))
    assert e.value.status == sgns.EINVAL
    with pytest.raises(sgns.SgnsError) as e:
        sgns.info_walks(ip, ix, cn, 4, 0, 5, 0.9, 1, trace=2)
    assert e.value.status == sgns.EINVAL
    for kw in (dict(max_length=0), dict(max_length=1001), dict(min_length=-1)):
        args = dict(min_length=0, max_length=5)
        args.update(kw)
        with pytest.raises(sgns.SgnsError) as e:
            sgns.info_walks(ip, ix, cn, 4, args["min_length"], args["max_length"], 0.9, 1)
        assert e.value.status == sgns.EINVAL
