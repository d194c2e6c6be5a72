"""Seeded synthetic graphs and walk corpora in the reference's formats.

The reference trains on walks its engine produces over real graphs (LiveJournal etc.,
not shipped).  These generators stand in for them with the shapes the benchmark
configurations name:
  * Chung-Lu power-law graphs (expected-degree model, weights (i + i0)^(-1/(gamma-1)));
  * k-block stochastic block models with a given p_in / p_out ratio;
  * a link-prediction holdout in the style of src/tools/gtrain.cpp:226-385 (remove test
    edges while both endpoints keep degree > 1, sample as many non-edges);
  * walk corpora: uniform random walks with fixed, geometric or uniform lengths, and
    information-oriented walks (the entropy/length correlation stop rule of
    include/walk.hpp:260-387, 868-874);
  * the in-memory corpus format (vertex ids, -1 after each walk; path.hpp:96,110) and the
    walk-file format (" %u" per vertex, newline per walk; path.hpp:92,108).
Every generator runs in torch on the given device, deterministically for a seed.
"""
import math

import numpy as np
import torch


def _gen(seed, device):
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    return g


def _csr_from_edges(src, dst, V):
    """Undirected simple graph: both directions, no self loops, no duplicates."""
    keep = src != dst
    src, dst = src[keep], dst[keep]
    a, b = torch.minimum(src, dst), torch.maximum(src, dst)
    key = torch.unique(a.long() * V + b.long())
    a, b = key // V, key % V
    u = torch.cat([a, b])
    v = torch.cat([b, a])
    order = torch.argsort(u * V + v)
    u, v = u[order], v[order]
    deg = torch.bincount(u, minlength=V)
    indptr = torch.zeros(V + 1, dtype=torch.int64, device=u.device)
    indptr[1:] = torch.cumsum(deg, 0)
    return indptr, v.to(torch.int32), key.numel()


def chung_lu(V, E, gamma=2.1, seed=1, device="cpu", i0=None):
    """Expected-degree power-law graph with about E undirected edges."""
    g = _gen(seed, device)
    if i0 is None:
        i0 = max(1.0, V ** 0.25)
    w = (torch.arange(V, dtype=torch.float64, device=device) + i0) ** (-1.0 / (gamma - 1.0))
    cdf = torch.cumsum(w / w.sum(), 0)
    cdf[-1] = 1.0
    want = int(E * 1.08) + 16
    u = torch.searchsorted(cdf, torch.rand(want, generator=g, dtype=torch.float64, device=device))
    v = torch.searchsorted(cdf, torch.rand(want, generator=g, dtype=torch.float64, device=device))
    u = u.clamp_max(V - 1)
    v = v.clamp_max(V - 1)
    indptr, indices, m = _csr_from_edges(u, v, V)
    return indptr, indices


def sbm(V, E, blocks=4, ratio=20.0, seed=1, device="cpu"):
    """k equal blocks; an edge is within a block with the probability the p_in/p_out
    ratio implies for equal-size blocks.  Returns (indptr, indices, block_of)."""
    g = _gen(seed, device)
    bs = V // blocks
    block_of = torch.clamp(torch.arange(V, device=device) // bs, max=blocks - 1)
    within_pairs = blocks * bs * bs / 2.0
    between_pairs = blocks * (blocks - 1) / 2.0 * bs * bs
    p_within = ratio * within_pairs / (ratio * within_pairs + between_pairs)
    want = int(E * 1.05) + 16
    inside = torch.rand(want, generator=g, device=device) < p_within
    b1 = torch.randint(0, blocks, (want,), generator=g, device=device)
    off = torch.randint(1, blocks, (want,), generator=g, device=device)
    b2 = torch.where(inside, b1, (b1 + off) % blocks)
    u = b1 * bs + torch.randint(0, bs, (want,), generator=g, device=device)
    v = b2 * bs + torch.randint(0, bs, (want,), generator=g, device=device)
    indptr, indices, m = _csr_from_edges(u, v, V)
    return indptr, indices, block_of


def edge_list(indptr, indices):
    V = indptr.numel() - 1
    deg = indptr[1:] - indptr[:-1]
    src = torch.repeat_interleave(torch.arange(V, device=indptr.device), deg)
    dst = indices.long()
    keep = src < dst
    return src[keep], dst[keep]


def holdout(indptr, indices, frac=0.1, seed=7):
    """Split off a fraction of the undirected edges for link prediction, keeping every
    endpoint's remaining degree > 1, and sample as many non-edges (gtrain.cpp:293-333).
    Returns (train_indptr, train_indices, test_pos[2, m], test_neg[2, m])."""
    dev = indptr.device
    g = _gen(seed, dev)
    V = indptr.numel() - 1
    src, dst = edge_list(indptr, indices)
    m = src.numel()
    want = int(m * frac)
    perm = torch.randperm(m, generator=g, device=dev)
    deg = indptr[1:] - indptr[:-1]
    cand = perm[: min(m, int(want * 1.5) + 16)]
    cs, cd = src[cand], dst[cand]
    # a candidate is removed when, counting every earlier candidate at each endpoint as
    # removed too, both endpoints keep degree > 1 (a conservative, vectorised form of the
    # sequential rule)
    ends = torch.cat([cs, cd])
    pos_in = torch.arange(ends.numel(), device=dev)
    order = torch.argsort(ends * ends.numel() + pos_in % cand.numel())
    sorted_ends = ends[order]
    first_of_run = torch.ones_like(sorted_ends, dtype=torch.bool)
    first_of_run[1:] = sorted_ends[1:] != sorted_ends[:-1]
    run_start = torch.cummax(torch.where(first_of_run, torch.arange(ends.numel(), device=dev),
                                         torch.zeros_like(pos_in)), 0).values
    rank_sorted = torch.arange(ends.numel(), device=dev) - run_start
    rank = torch.empty_like(rank_sorted)
    rank[order] = rank_sorted
    ra, rb = rank[: cand.numel()], rank[cand.numel():]
    ok = (deg[cs] - ra > 2) & (deg[cd] - rb > 2)
    removed = ok & (torch.cumsum(ok.long(), 0) <= want)
    test_ids = cand[removed]
    keep = torch.ones(m, dtype=torch.bool, device=dev)
    keep[test_ids] = False
    tr_indptr, tr_indices, _ = _csr_from_edges(src[keep], dst[keep], V)
    pos = torch.stack([src[test_ids], dst[test_ids]])
    # non-edges: uniform pairs not in the full graph
    have = set((src * V + dst).tolist()) if m < 5_000_000 else None
    neg_u, neg_v = [], []
    need = pos.shape[1]
    while need > 0:
        a = torch.randint(0, V, (need * 2,), generator=g, device=dev)
        b = torch.randint(0, V, (need * 2,), generator=g, device=dev)
        lo, hi = torch.minimum(a, b), torch.maximum(a, b)
        ok = lo != hi
        lo, hi = lo[ok], hi[ok]
        if have is not None:
            keys = (lo * V + hi).tolist()
            mask = torch.tensor([k not in have for k in keys], dtype=torch.bool, device=dev)
        else:
            full = torch.sort(src * V + dst).values
            kk = lo * V + hi
            idx = torch.searchsorted(full, kk).clamp_max(full.numel() - 1)
            mask = full[idx] != kk
        lo, hi = lo[mask][:need], hi[mask][:need]
        neg_u.append(lo)
        neg_v.append(hi)
        need -= lo.numel()
    neg = torch.stack([torch.cat(neg_u), torch.cat(neg_v)])
    return tr_indptr, tr_indices, pos, neg


def walk_lengths(n, kind="fixed", length=80, mean=40, cap=80, lo=5, hi=200, seed=3, device="cpu"):
    g = _gen(seed, device)
    if kind == "fixed":
        return torch.full((n,), int(length), dtype=torch.int64, device=device)
    if kind == "geometric":  # support 1, 2, ... with the given mean, capped
        p = 1.0 / mean
        u = torch.rand(n, generator=g, dtype=torch.float64, device=device).clamp_min(1e-300)
        L = torch.floor(torch.log(u) / math.log(1.0 - p)).long() + 1
        return L.clamp(1, cap)
    if kind == "uniform":
        return torch.randint(lo, hi + 1, (n,), generator=g, device=device)
    raise ValueError(kind)


def random_walks(indptr, indices, walks_per_vertex=10, lengths=None, seed=5, device=None):
    """Uniform random walks, walks_per_vertex rounds over a shuffled vertex order.
    lengths: int64 tensor (one per walk, in output order) or an int.  Returns the
    corpus (int32, -1 after each walk) on the graph's device."""
    dev = indptr.device if device is None else device
    indptr, indices = indptr.to(dev), indices.to(dev)
    g = _gen(seed, dev)
    V = indptr.numel() - 1
    starts = torch.cat([torch.randperm(V, generator=g, device=dev) for _ in range(walks_per_vertex)])
    n = starts.numel()
    if lengths is None:
        lengths = 80
    if isinstance(lengths, int):
        lengths = torch.full((n,), lengths, dtype=torch.int64, device=dev)
    lengths = lengths.to(dev)
    Lmax = int(lengths.max())
    deg = indptr[1:] - indptr[:-1]
    walks = torch.empty((n, Lmax), dtype=torch.int32, device=dev)
    cur = starts.long()
    walks[:, 0] = cur.to(torch.int32)
    for t in range(1, Lmax):
        dc = deg[cur]
        r = torch.rand(n, generator=g, device=dev, dtype=torch.float64)
        off = torch.floor(r * dc.to(torch.float64)).long().clamp_max((dc - 1).clamp_min(0))
        nxt = indices[(indptr[cur] + off).clamp_max(indices.numel() - 1)].long()
        cur = torch.where(dc > 0, nxt, cur)
        walks[:, t] = cur.to(torch.int32)
    # isolated start vertices: walk of length 1
    lengths = torch.where(deg[starts] > 0, lengths, torch.ones_like(lengths))
    col = torch.arange(Lmax + 1, device=dev)
    out = torch.full((n, Lmax + 1), -2, dtype=torch.int32, device=dev)
    out[:, :Lmax] = walks
    out[col.unsqueeze(0) >= lengths.unsqueeze(1)] = -2
    out[torch.arange(n, device=dev), lengths] = -1
    flat = out.reshape(-1)
    return flat[flat != -2]


def information_walks(indptr, indices, walks_per_vertex=10, min_length=20, max_length=80, r_min=0.995,
                      seed=5, device=None):
    """Walks that stop once the correlation R between the walk's path entropy H_n and its
    length S_n satisfies R^2 < r_min or R < 0, after min_length steps (the
    information-oriented rule of include/walk.hpp:284-354, 868-874), capped at max_length.
    H_n is the Shannon entropy (bits) of the walk's vertex-visit frequencies, updated
    incrementally from the current vertex's previous count as Correlation::iterateHn
    does; the running moments follow Correlation::iterate."""
    dev = indptr.device if device is None else device
    indptr, indices = indptr.to(dev), indices.to(dev)
    g = _gen(seed, dev)
    V = indptr.numel() - 1
    starts = torch.cat([torch.randperm(V, generator=g, device=dev) for _ in range(walks_per_vertex)])
    n = starts.numel()
    deg = indptr[1:] - indptr[:-1]
    walks = torch.empty((n, max_length), dtype=torch.int32, device=dev)
    cur = starts.long()
    walks[:, 0] = cur.to(torch.int32)
    alive = torch.ones(n, dtype=torch.bool, device=dev)
    length = torch.ones(n, dtype=torch.int64, device=dev)
    f64 = torch.float64
    T = torch.zeros(n, dtype=f64, device=dev)  # sum_k c_k log2 c_k over visited vertices
    EH = torch.zeros(n, dtype=f64, device=dev)
    ES = torch.ones(n, dtype=f64, device=dev)
    EHS = torch.zeros(n, dtype=f64, device=dev)
    EHH = torch.zeros(n, dtype=f64, device=dev)
    ESS = torch.ones(n, dtype=f64, device=dev)
    N = torch.ones(n, dtype=f64, device=dev)

    def xlog2x(c):
        return torch.where(c > 0, c * torch.log2(c.clamp_min(1.0)), torch.zeros_like(c))

    for t in range(1, max_length):
        if not bool(alive.any()):
            break
        dc = deg[cur]
        r = torch.rand(n, generator=g, device=dev, dtype=f64)
        off = torch.floor(r * dc.to(f64)).long().clamp_max((dc - 1).clamp_min(0))
        nxt = indices[(indptr[cur] + off).clamp_max(indices.numel() - 1)].long()
        cur = torch.where((dc > 0) & alive, nxt, cur)
        walks[:, t] = cur.to(torch.int32)
        prev = (walks[:, :t] == cur.to(torch.int32).unsqueeze(1)).sum(1).to(f64)
        T = torch.where(alive, T + xlog2x(prev + 1) - xlog2x(prev), T)
        length = torch.where(alive, length + 1, length)
        S = length.to(f64)
        H = torch.log2(S) - T / S
        N1 = N + 1
        upd = alive
        EH = torch.where(upd, EH + (H - EH) / N1, EH)
        ES = torch.where(upd, ES + (S - ES) / N1, ES)
        EHS = torch.where(upd, EHS + (H * S - EHS) / N1, EHS)
        EHH = torch.where(upd, EHH + (H * H - EHH) / N1, EHH)
        ESS = torch.where(upd, ESS + (S * S - ESS) / N1, ESS)
        N = torch.where(upd, N1, N)
        DH = (EHH - EH * EH).clamp_min(1e-300)
        DS = (ESS - ES * ES).clamp_min(1e-300)
        R = (EHS - EH * ES) / torch.sqrt(DH * DS)
        stop = alive & (length > min_length) & ((R * R < r_min) | (R < 0))
        alive = alive & ~stop
    lengths = length
    Lmax = walks.shape[1]
    col = torch.arange(Lmax + 1, device=dev)
    out = torch.full((n, Lmax + 1), -2, dtype=torch.int32, device=dev)
    out[:, :Lmax] = walks
    out[col.unsqueeze(0) >= lengths.unsqueeze(1)] = -2
    out[torch.arange(n, device=dev), lengths] = -1
    flat = out.reshape(-1)
    return flat[flat != -2]


# ---- platform-independent generators (numpy integer arithmetic only) ----------------
# The same seed gives the same graph, holdout and pairs on every host (x86 and Arm alike),
# so a corpus drawn from them on the GPU can be compared with one a CPU trainer used.
_G = np.uint64(0x9E3779B97F4A7C15)


def _mix64(z):
    """SplitMix64 finaliser (Steele, Lea, Flood 2014) on a uint64 array, adding G first."""
    with np.errstate(over="ignore"):
        z = np.asarray(z, dtype=np.uint64) + _G
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def _stream(seed, purpose, n):
    """n uint64 draws of the stream (seed, purpose)."""
    with np.errstate(over="ignore"):
        base = _mix64(np.uint64(seed) ^ (np.uint64(purpose) * _G))
        return _mix64(base + np.arange(n, dtype=np.uint64) * _G)


def _below(r, n):
    """Lemire's multiply-shift: uniform integers in [0, n) from 64-bit draws (high 32 bits)."""
    return ((r >> np.uint64(32)) * np.uint64(n)) >> np.uint64(32)


def _csr_from_pairs_np(a, b, V):
    """Undirected simple graph from pairs: no self loops, no duplicates, sorted lists."""
    keep = a != b
    a, b = a[keep], b[keep]
    lo, hi = np.minimum(a, b).astype(np.int64), np.maximum(a, b).astype(np.int64)
    key = np.unique(lo * V + hi)
    lo, hi = key // V, key % V
    u = np.concatenate([lo, hi])
    v = np.concatenate([hi, lo])
    order = np.argsort(u * V + v, kind="stable")
    u, v = u[order], v[order]
    indptr = np.zeros(V + 1, np.int64)
    np.cumsum(np.bincount(u, minlength=V), out=indptr[1:])
    return indptr, v.astype(np.int32)


def sbm_csr(V, E, blocks=4, ratio=20.0, seed=1):
    """k equal blocks of consecutive vertex ids; a candidate edge lies within a block with
    the probability the p_in / p_out ratio gives for equal blocks.  About E undirected
    edges (duplicates and self pairs of the int(1.05 E) candidates are dropped).
    Returns (indptr int64 [V + 1], indices int32, block_of int32 [V])."""
    bs = V // blocks
    block_of = np.minimum(np.arange(V) // bs, blocks - 1).astype(np.int32)
    within = blocks * bs * bs / 2.0
    between = blocks * (blocks - 1) / 2.0 * bs * bs
    p_within = ratio * within / (ratio * within + between)
    n = int(E * 1.05) + 16
    thr = np.uint64(int(p_within * 2.0 ** 53))
    inside = (_stream(seed, 1, n) >> np.uint64(11)) < thr
    b1 = _below(_stream(seed, 2, n), blocks).astype(np.int64)
    off = 1 + _below(_stream(seed, 3, n), blocks - 1).astype(np.int64)
    b2 = np.where(inside, b1, (b1 + off) % blocks)
    u = b1 * bs + _below(_stream(seed, 4, n), bs).astype(np.int64)
    v = b2 * bs + _below(_stream(seed, 5, n), bs).astype(np.int64)
    indptr, indices = _csr_from_pairs_np(u, v, V)
    return indptr, indices, block_of


def holdout_csr(indptr, indices, frac=0.1, seed=7):
    """The link-prediction split of src/tools/gtrain.cpp:293-333: edges are visited in a
    seeded random order and removed while both endpoints still have degree > 1, until
    frac of the undirected edges are removed; as many non-edges (distinct pairs u != v that
    are not edges of the full graph) are sampled.  Returns (train_indptr, train_indices,
    pos [2, m] int64, neg [2, m] int64)."""
    V = len(indptr) - 1
    deg = np.diff(indptr).astype(np.int64)
    src = np.repeat(np.arange(V, dtype=np.int64), deg)
    dst = indices.astype(np.int64)
    keep = src < dst
    src, dst = src[keep], dst[keep]
    m = len(src)
    want = int(m * frac)
    order = np.argsort(_stream(seed, 11, m), kind="stable")
    d = deg.copy()
    removed = np.zeros(m, bool)
    got = 0
    so, do = src[order].tolist(), dst[order].tolist()
    dl = d.tolist()
    for i in range(m):
        if got >= want:
            break
        a, b = so[i], do[i]
        if dl[a] > 1 and dl[b] > 1:
            dl[a] -= 1
            dl[b] -= 1
            removed[order[i]] = True
            got += 1
    tr_indptr, tr_indices = _csr_from_pairs_np(src[~removed], dst[~removed], V)
    pos = np.stack([src[removed], dst[removed]])
    full = np.sort(src * V + dst)
    neg_keys = np.zeros(0, np.int64)
    k = 0
    while len(neg_keys) < got:
        n = 2 * (got - len(neg_keys)) + 64
        a = _below(_stream(seed, 100 + 2 * k, n), V).astype(np.int64)
        b = _below(_stream(seed, 101 + 2 * k, n), V).astype(np.int64)
        k += 1
        lo, hi = np.minimum(a, b), np.maximum(a, b)
        ok = lo != hi
        kk = (lo * V + hi)[ok]
        idx = np.searchsorted(full, kk).clip(max=len(full) - 1)
        kk = kk[full[idx] != kk]
        # keep first occurrences, in draw order, of pairs not drawn before
        _, first = np.unique(kk, return_index=True)
        kk = kk[np.sort(first)]
        kk = kk[~np.isin(kk, neg_keys)]
        neg_keys = np.concatenate([neg_keys, kk])[:got]
    neg = np.stack([neg_keys // V, neg_keys % V])
    return tr_indptr, tr_indices, pos, neg


def vertex_counts(corpus, V):
    """Per-vertex occurrence counts of a corpus (the reference's vertex_cn, path.hpp:98)."""
    c = torch.as_tensor(corpus)
    c = c[c >= 0].long()
    return torch.bincount(c, minlength=V).to(torch.int32)


def write_walk_file(corpus, path):
    """One walk per line, " %u" per vertex (path.hpp:92,108)."""
    c = np.asarray(torch.as_tensor(corpus).cpu().numpy(), dtype=np.int64)
    ends = np.flatnonzero(c == -1)
    with open(path, "w") as f:
        start = 0
        for e in ends:
            f.write("".join(" %d" % v for v in c[start:e]) + "\n")
            start = e + 1


def link_auc(emb, pos, neg):
    """AUC of dot-product scores of held-out edges against sampled non-edges.
    emb: [V, d] in vertex-id order."""
    e = torch.as_tensor(emb, dtype=torch.float32)
    pos, neg = torch.as_tensor(pos).long().cpu(), torch.as_tensor(neg).long().cpu()
    e = e.cpu()
    sp = (e[pos[0]] * e[pos[1]]).sum(1)
    sn = (e[neg[0]] * e[neg[1]]).sum(1)
    return auc_from_scores(sp, sn)


def link_auc_device(trainer, pos, neg):
    """The same AUC with the scores computed on the GPU by sgns_link_scores from the
    trainer's input table (rows in sorted order; vertex ids mapped through its order)."""
    import sgns

    order = torch.as_tensor(trainer.order().astype(np.int64))
    row_of = torch.empty_like(order)
    row_of[order] = torch.arange(order.numel())
    V, d = order.numel(), trainer.opt.size
    wih, _ = trainer.device_tables()
    dtype = 1 if trainer.opt.storage == sgns.STORE_BF16_SR else 0
    out = []
    for p in (pos, neg):
        p = torch.as_tensor(p).long().cpu()
        pairs = torch.stack([row_of[p[0]], row_of[p[1]]], 1).to(torch.int32).cuda()
        sc = torch.empty(pairs.shape[0], dtype=torch.float32, device="cuda")
        sgns.link_scores(dtype, d, wih, V, pairs, sc)
        out.append(sc)
    return auc_from_scores(out[0], out[1])


def auc_from_scores(sp, sn):
    """Mann-Whitney AUC of positive scores sp against negative scores sn (ties averaged),
    in fp64 on the scores' device."""
    scores = torch.cat([sp, sn]).double()
    labels = torch.cat([torch.ones_like(sp), torch.zeros_like(sn)]).double()
    order = torch.argsort(scores)
    ranks = torch.empty_like(scores)
    ranks[order] = torch.arange(1, scores.numel() + 1, dtype=torch.float64, device=scores.device)
    # average ranks of ties
    s_sorted = scores[order]
    uniq, inv, cnt = torch.unique_consecutive(s_sorted, return_inverse=True, return_counts=True)
    csum = torch.cumsum(cnt, 0).double()
    avg = csum - (cnt.double() - 1) / 2
    ranks[order] = avg[inv]
    npos, nneg = float(sp.numel()), float(sn.numel())
    return float((ranks[labels == 1].sum() - npos * (npos + 1) / 2) / (npos * nneg))
