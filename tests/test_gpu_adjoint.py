"""The hand-written SGNS adjoint through the C ABI, wrapped in a test-only
torch.autograd.Function, against finite differences (fp64, eps = 1e-6) and the fp64
autograd gradient of the same loss written in plain torch."""
import numpy as np
import pytest

import sgns

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def sbm_minibatches(V=1000, n=64, K=5, w=5, seed=3):
    """Minibatches with the reference step's layout, drawn from walks on an SBM slice."""
    import synth

    ip, ix, _ = synth.sbm(V, 6 * V, seed=seed)
    corpus = synth.random_walks(ip, ix, 1, 30, seed=seed + 1).numpy()
    walks = np.split(corpus, np.flatnonzero(corpus == -1) + 1)[:-1]
    walks = [x[:-1] for x in walks if len(x) > 3]
    rng = np.random.default_rng(seed)
    in_ids, in_ptr, first, out_ids, out_ptr, meta = [], [0], [], [], [0], []
    for b in range(n):
        w1, w2 = walks[rng.integers(len(walks))], walks[rng.integers(len(walks))]
        p1, p2 = rng.integers(len(w1)), rng.integers(len(w2))
        c1 = [w1[c] for c in range(max(0, p1 - w), min(len(w1), p1 + w + 1)) if c != p1]
        c2 = [w2[c] for c in range(max(0, p2 - w), min(len(w2), p2 + w + 1)) if c != p2]
        negs = rng.integers(0, V, K)
        outs, mt = [w1[p1]], [1]
        for s in negs:
            if s in outs:
                mt[outs.index(s)] += 1 if outs.index(s) > 0 else 0
            else:
                outs.append(s)
                mt.append(1)
        outs.append(w2[p2])
        mt.append(1)
        in_ids += c1 + c2
        in_ptr.append(len(in_ids))
        first.append(len(c1))
        out_ids += outs
        out_ptr.append(len(out_ids))
        meta += mt
    dev = "cuda"
    as_t = lambda a: torch.tensor(np.asarray(a, dtype=np.int32), device=dev)
    return dict(in_ptr=as_t(in_ptr), in_ids=as_t(in_ids), in_first=as_t(first), out_ptr=as_t(out_ptr),
                out_ids=as_t(out_ids), out_meta=as_t(meta), V=V)


class SgnsLoss(torch.autograd.Function):
    """loss(Wih, Woh) over fixed minibatches; backward = the library's sparse adjoint."""

    @staticmethod
    def forward(ctx, wih, woh, mb):
        dtype = 2 if wih.dtype == torch.float64 else 0
        d = wih.shape[1]
        n_in, n_out = mb["in_ids"].numel(), mb["out_ids"].numel()
        loss = torch.zeros(1, dtype=torch.float64, device=wih.device)
        gi_ids = torch.empty(n_in, dtype=torch.int32, device=wih.device)
        go_ids = torch.empty(n_out, dtype=torch.int32, device=wih.device)
        gi = torch.empty((n_in, d), dtype=wih.dtype, device=wih.device)
        go = torch.empty((n_out, d), dtype=wih.dtype, device=wih.device)
        ni, no = sgns.loss_adjoint(dtype, d, mb["V"], mb["in_ptr"], mb["in_ids"], mb["in_first"], mb["out_ptr"],
                                   mb["out_ids"], mb["out_meta"], wih.contiguous().data_ptr(),
                                   woh.contiguous().data_ptr(), loss, gi_ids, gi, go_ids, go,
                                   stream=torch.cuda.current_stream().cuda_stream)
        ctx.save_for_backward(gi_ids[:ni].long(), gi[:ni], go_ids[:no].long(), go[:no])
        ctx.shapes = (wih.shape, woh.shape)
        return loss.to(wih.dtype).reshape(())

    @staticmethod
    def backward(ctx, g):
        gi_ids, gi, go_ids, go = ctx.saved_tensors
        sw, so = ctx.shapes
        dw = torch.zeros(sw, dtype=gi.dtype, device=gi.device).index_add_(0, gi_ids, gi) * g
        do = torch.zeros(so, dtype=go.dtype, device=go.device).index_add_(0, go_ids, go) * g
        return dw, do, None


def torch_loss(wih, woh, mb):
    """The same loss in plain torch (fp64 autograd reference)."""
    loss = 0
    ip, op = mb["in_ptr"].tolist(), mb["out_ptr"].tolist()
    ii, oo, ff, mm = mb["in_ids"].long(), mb["out_ids"].long(), mb["in_first"].tolist(), mb["out_meta"]
    for b in range(len(ff)):
        x = wih[ii[ip[b]:ip[b + 1]]]
        o = woh[oo[op[b]:op[b + 1]]]
        f = o @ x.T
        O, I = f.shape
        lab = torch.zeros_like(f)
        lab[0, :ff[b]] = 1
        lab[O - 1, ff[b]:] = 1
        m = mm[op[b]:op[b + 1]].to(f.dtype).unsqueeze(1)
        loss = loss + (m * torch.nn.functional.softplus(-(2 * lab - 1) * f)).sum()
    return loss


def tables(V, d, dtype, seed=0):
    g = torch.Generator(device="cuda").manual_seed(seed)
    wih = (torch.rand((V, d), generator=g, device="cuda", dtype=dtype) - 0.5) * 0.5
    woh = (torch.rand((V, d), generator=g, device="cuda", dtype=dtype) - 0.5) * 0.5
    return wih, woh


def test_adjoint_matches_fp64_autograd(sgns_lib):
    mb = sbm_minibatches()
    wih, woh = tables(mb["V"], 32, torch.float64)
    a = wih.clone().requires_grad_(True)
    b = woh.clone().requires_grad_(True)
    L = SgnsLoss.apply(a, b, mb)
    L.backward()
    a2 = wih.clone().requires_grad_(True)
    b2 = woh.clone().requires_grad_(True)
    L2 = torch_loss(a2, b2, mb)
    L2.backward()
    assert abs(L.item() - L2.item()) <= 1e-12 * abs(L2.item())
    assert torch.allclose(a.grad, a2.grad, rtol=1e-10, atol=1e-13)
    assert torch.allclose(b.grad, b2.grad, rtol=1e-10, atol=1e-13)


def test_adjoint_finite_differences(sgns_lib):
    mb = sbm_minibatches(n=16)
    wih, woh = tables(mb["V"], 32, torch.float64, seed=1)
    a = wih.clone().requires_grad_(True)
    b = woh.clone().requires_grad_(True)
    assert torch.autograd.gradcheck(lambda x, y: SgnsLoss.apply(x, y, mb), (a, b), eps=1e-6, atol=1e-5, rtol=1e-3,
                                    fast_mode=True)
    # central differences on touched coordinates
    L = SgnsLoss.apply(a, b, mb)
    L.backward()
    rng = np.random.default_rng(0)
    rows_in = mb["in_ids"].long().unique().tolist()
    rows_out = mb["out_ids"].long().unique().tolist()
    eps = 1e-6
    for tab, grad, rows in ((wih, a.grad, rows_in), (woh, b.grad, rows_out)):
        for _ in range(40):
            r, c = int(rng.choice(rows)), int(rng.integers(32))
            tp, tm = tab.clone(), tab.clone()
            tp[r, c] += eps
            tm[r, c] -= eps
            if tab is wih:
                fp, fm = SgnsLoss.apply(tp, woh, mb).item(), SgnsLoss.apply(tm, woh, mb).item()
            else:
                fp, fm = SgnsLoss.apply(wih, tp, mb).item(), SgnsLoss.apply(wih, tm, mb).item()
            fd = (fp - fm) / (2 * eps)
            assert abs(fd - grad[r, c].item()) <= 1e-6 + 1e-5 * abs(fd), (r, c, fd, grad[r, c].item())


def test_adjoint_fp32_close_to_fp64(sgns_lib):
    mb = sbm_minibatches(n=128, seed=9)
    w64, o64 = tables(mb["V"], 32, torch.float64, seed=2)
    a = w64.clone().requires_grad_(True)
    b = o64.clone().requires_grad_(True)
    SgnsLoss.apply(a, b, mb).backward()
    a32 = w64.float().requires_grad_(True)
    b32 = o64.float().requires_grad_(True)
    L32 = SgnsLoss.apply(a32, b32, mb)
    L32.backward()
    rel = (a32.grad.double() - a.grad).norm() / a.grad.norm()
    assert rel < 1e-5, rel


def test_sparse_rows_ascending_and_unique(sgns_lib):
    mb = sbm_minibatches(n=32, seed=4)
    wih, woh = tables(mb["V"], 32, torch.float32, seed=3)
    d = 32
    n_in, n_out = mb["in_ids"].numel(), mb["out_ids"].numel()
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    gi_ids = torch.empty(n_in, dtype=torch.int32, device="cuda")
    go_ids = torch.empty(n_out, dtype=torch.int32, device="cuda")
    gi = torch.empty((n_in, d), device="cuda")
    go = torch.empty((n_out, d), device="cuda")
    ni, no = sgns.loss_adjoint(0, d, mb["V"], mb["in_ptr"], mb["in_ids"], mb["in_first"], mb["out_ptr"],
                               mb["out_ids"], mb["out_meta"], wih.data_ptr(), woh.data_ptr(), loss, gi_ids, gi,
                               go_ids, go)
    ids = gi_ids[:ni].cpu().numpy()
    assert ni == len(np.unique(mb["in_ids"].cpu().numpy())) and (np.diff(ids) > 0).all()
    ids = go_ids[:no].cpu().numpy()
    assert no == len(np.unique(mb["out_ids"].cpu().numpy())) and (np.diff(ids) > 0).all()


def dense_adjoint(code, wih, woh, mb):
    """loss and dense (fp64) gradients from the library's sparse adjoint; code = table type
    (0 fp32, 1 bf16, 2 fp64)."""
    d = wih.shape[1]
    gdt = torch.float64 if code == 2 else torch.float32
    n_in, n_out = mb["in_ids"].numel(), mb["out_ids"].numel()
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    gi_ids = torch.empty(n_in, dtype=torch.int32, device="cuda")
    go_ids = torch.empty(n_out, dtype=torch.int32, device="cuda")
    gi = torch.empty((n_in, d), dtype=gdt, device="cuda")
    go = torch.empty((n_out, d), dtype=gdt, device="cuda")
    ni, no = sgns.loss_adjoint(code, d, mb["V"], mb["in_ptr"], mb["in_ids"], mb["in_first"], mb["out_ptr"],
                               mb["out_ids"], mb["out_meta"], wih.data_ptr(), woh.data_ptr(), loss, gi_ids, gi,
                               go_ids, go)
    dw = torch.zeros(wih.shape, dtype=torch.float64, device="cuda").index_add_(0, gi_ids[:ni].long(),
                                                                               gi[:ni].double())
    do = torch.zeros(woh.shape, dtype=torch.float64, device="cuda").index_add_(0, go_ids[:no].long(),
                                                                               go[:no].double())
    return loss.item(), dw, do


# (table type, d, negatives, window): rows of whole 16-byte chunks take the pipelined
# kernel (up to 40 inputs and 12 outputs per minibatch, rows of 4 to 64 chunks; bf16 rows
# on the tensor cores, d = 24 with a half-width last column block); d = 36 bf16 (72-byte
# rows) and d = 30 fp32 take the general one
@pytest.mark.parametrize("code,d,K,w", [(1, 128, 5, 10), (1, 256, 10, 10), (1, 24, 10, 10), (0, 256, 10, 5),
                                        (0, 64, 5, 10), (2, 32, 10, 10), (1, 36, 5, 10), (0, 30, 5, 5)])
def test_adjoint_kernels_against_fp64_autograd(sgns_lib, code, d, K, w):
    mb = sbm_minibatches(n=48, K=K, w=w, seed=11 + d + K)
    dt = {0: torch.float32, 1: torch.bfloat16, 2: torch.float64}[code]
    w64, o64 = tables(mb["V"], d, torch.float64, seed=5)
    wih, woh = w64.to(dt), o64.to(dt)
    loss, dw, do = dense_adjoint(code, wih, woh, mb)
    a = wih.double().requires_grad_(True)
    b = woh.double().requires_grad_(True)
    ref = torch_loss(a, b, mb)
    ref.backward()
    tol = 1e-12 if code == 2 else 2e-6
    assert abs(loss - ref.item()) <= tol * abs(ref.item())
    for got, want in ((dw, a.grad), (do, b.grad)):
        err = (got - want).abs().max().item()
        assert err <= tol * want.abs().max().item() * 10, (err, want.abs().max().item())
