"""Per-minibatch update of the GPU step code against the oracle step.

fp32: bit for bit with the oracle's fused sequential order.  Against an fp64 oracle the
per-row relative error of the update stays within 1e-5 (the tolerance of the plain fp32
form under Hogwild ordering), except for pairs whose dot product sits on a sigmoid-table
cell boundary, where the table value itself changes (counted and bounded below)."""
import numpy as np
import pytest

import sgns

pytestmark = pytest.mark.gpu


def random_minibatches(n, d, seed, scale=0.3):
    rng = np.random.default_rng(seed)
    batches = []
    for _ in range(n):
        I = int(rng.integers(2, 41))
        first = int(rng.integers(1, I))
        O = int(rng.integers(2, 13))
        meta = np.ones(O, np.int32)
        meta[1:O - 1] = rng.integers(1, 4, O - 2)
        xin = (rng.standard_normal((I, d)) * scale / np.sqrt(d)).astype(np.float32)
        xout = (rng.standard_normal((O, d)) * scale).astype(np.float32)
        alpha = np.float32(rng.uniform(1e-4, 0.05))
        batches.append((xin, xout, meta, first, alpha))
    return batches


def run_gpu(batches, d):
    import torch

    dev = "cuda"
    in_count = torch.tensor([b[0].shape[0] for b in batches], dtype=torch.int32, device=dev)
    in_first = torch.tensor([b[3] for b in batches], dtype=torch.int32, device=dev)
    out_count = torch.tensor([b[1].shape[0] for b in batches], dtype=torch.int32, device=dev)
    meta = torch.tensor(np.concatenate([b[2] for b in batches]), device=dev)
    alpha = torch.tensor([b[4] for b in batches], dtype=torch.float32, device=dev)
    xin = torch.tensor(np.concatenate([b[0] for b in batches]), device=dev)
    xout = torch.tensor(np.concatenate([b[1] for b in batches]), device=dev)
    d_in = torch.full_like(xin, float("nan"))
    d_out = torch.full_like(xout, float("nan"))
    sgns.minibatch_update(d, in_count, in_first, out_count, meta, alpha, xin, xout, d_in, d_out,
                          stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return d_in.cpu().numpy(), d_out.cpu().numpy()


@pytest.mark.parametrize("d", [16, 64, 128, 256, 100])
def test_minibatch_bit_exact_vs_oracle(d, sgns_lib, oracle_mod):
    batches = random_minibatches(200, d, seed=d)
    gi, go = run_gpu(batches, d)
    oi = oo = 0
    for xin, xout, meta, first, alpha in batches:
        dIn, dOut = oracle_mod.minibatch(xin, xout, meta, first, float(alpha), acc64=False)
        I, O = xin.shape[0], xout.shape[0]
        assert np.array_equal(gi[oi:oi + I], dIn.astype(np.float32))
        assert np.array_equal(go[oo:oo + O], dOut.astype(np.float32))
        oi += I
        oo += O


def test_minibatch_error_vs_fp64(sgns_lib, oracle_mod):
    d = 128
    batches = random_minibatches(1000, d, seed=5)
    gi, go = run_gpu(batches, d)
    oi = oo = 0
    errs, flips = [], 0
    for xin, xout, meta, first, alpha in batches:
        dIn, dOut = oracle_mod.minibatch(xin, xout, meta, first, float(alpha), acc64=True)
        I, O = xin.shape[0], xout.shape[0]
        for got, ref in ((gi[oi:oi + I], dIn), (go[oo:oo + O], dOut)):
            num = np.linalg.norm(got - ref, axis=1)
            den = np.maximum(np.linalg.norm(ref, axis=1), 1e-30)
            e = num / den
            if (e > 1e-5).any():
                flips += 1
            errs.append(e.max())
        oi += I
        oo += O
    errs = np.array(errs)
    # sigma-table cell crossings are rare; all other rows are within 1e-5
    assert flips <= 0.02 * len(errs), flips
    assert np.median(errs) < 1e-6


M64 = (1 << 64) - 1


def mix64(z):
    z = (z + 0x9E3779B97F4A7C15) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


M32 = (1 << 32) - 1


def fmix32(h):
    h ^= h >> 16
    h = (h * 0x7FEB352D) & M32
    h ^= h >> 15
    h = (h * 0x846CA68B) & M32
    return h ^ (h >> 16)


def sr_bits4(key, r, q):
    """64 bits for columns 4q..4q+3 of row r: h = fmix32(lo32(key) ^ (r * 0x9E3779B1 +
    q * 0x85EBCA77)), t = (h ^ hi32(key)) * 0x9E3779B1 mod 2^32, bits = (t ^ t >> 16) << 32 | h."""
    h = fmix32((key & M32) ^ ((r * 0x9E3779B1 + q * 0x85EBCA77) & M32))
    t = ((h ^ (key >> 32)) * 0x9E3779B1) & M32
    return ((t ^ (t >> 16)) << 32) | h


def sr_rows(v, seed, kind, b):
    """The trainers' write-back rule on fp32 rows v [rows, d]: column 4q + j of row r takes
    bits [16j, 16j + 16) of sr_bits4(key, r, q), key = mix64(seed ^ (kind << 56) ^ b);
    stored bits = (bits(x) + r16) >> 16."""
    key = mix64((seed ^ (kind << 56) ^ b) & M64)
    u = v.astype(np.float32).view(np.uint32).astype(np.uint64)
    out = np.zeros(v.shape, np.uint16)
    for r in range(v.shape[0]):
        for q in range(v.shape[1] // 4):
            bits = sr_bits4(key, r, q)
            for j in range(4):
                r16 = (bits >> (16 * j)) & 0xFFFF
                out[r, 4 * q + j] = (int(u[r, 4 * q + j]) + r16) >> 16
    return out


def run_gpu_bf16(batches, d, seed):
    import torch

    dev = "cuda"
    in_count = torch.tensor([b[0].shape[0] for b in batches], dtype=torch.int32, device=dev)
    in_first = torch.tensor([b[3] for b in batches], dtype=torch.int32, device=dev)
    out_count = torch.tensor([b[1].shape[0] for b in batches], dtype=torch.int32, device=dev)
    meta = torch.tensor(np.concatenate([b[2] for b in batches]), device=dev)
    alpha = torch.tensor([b[4] for b in batches], dtype=torch.float32, device=dev)
    xin = torch.tensor(np.concatenate([b[0] for b in batches]), device=dev)
    xout = torch.tensor(np.concatenate([b[1] for b in batches]), device=dev)
    n_in = torch.full(xin.shape, 0x7FC1, dtype=torch.int16, device=dev)
    n_out = torch.full(xout.shape, 0x7FC1, dtype=torch.int16, device=dev)
    sgns.minibatch_update_bf16(d, in_count, in_first, out_count, meta, alpha, xin, xout, n_in, n_out, seed)
    torch.cuda.synchronize()
    return n_in.cpu().numpy().view(np.uint16), n_out.cpu().numpy().view(np.uint16)


def bf16_values(batches):
    """The same minibatches with every row rounded to a bf16 value (a BF16 table's rows)."""
    r = lambda a: ((a.view(np.uint32) + 0x8000) & 0xFFFF0000).view(np.float32)
    return [(r(x), r(o), m, f, a) for x, o, m, f, a in batches]


@pytest.mark.parametrize("d", [16, 128, 256])
def test_bf16_writeback_is_the_trainers_rounding(d, sgns_lib):
    """sgns_minibatch_update_bf16 stores row + update (the fp32 update of
    sgns_minibatch_update, added in fp32) with the trainers' stochastic-rounding rule."""
    batches = bf16_values(random_minibatches(40, d, seed=100 + d))
    gi, go = run_gpu(batches, d)
    bi, bo = run_gpu_bf16(batches, d, seed=77)
    oi = oo = 0
    for b, (xin, xout, meta, first, alpha) in enumerate(batches):
        I, O = xin.shape[0], xout.shape[0]
        exp_in = sr_rows(xin + gi[oi:oi + I], 77, 2, b)    # inputs: event kind 2 (walk rows)
        exp_out = sr_rows(xout + go[oo:oo + O], 77, 4, b)  # outputs: event kind 4 (negatives)
        assert np.array_equal(bi[oi:oi + I], exp_in), b
        assert np.array_equal(bo[oo:oo + O], exp_out), b
        oi += I
        oo += O


def test_bf16_per_minibatch_error_vs_fp64(sgns_lib, oracle_mod):
    """Configuration 3's error statement at test size: 1000 minibatches from bf16 rows, each
    row's stored bf16 value against the fp64 step.  Stochastic rounding moves an element by
    less than one bf16 unit in the last place (2^-7 of its magnitude or less), so no row's
    relative error can exceed 2^-7; it is unbiased, so the mean signed error is near 0 ulp."""
    d = 128
    batches = bf16_values(random_minibatches(1000, d, seed=6))
    bi, bo = run_gpu_bf16(batches, d, seed=5)
    widen = lambda u: (u.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    ri, ro = widen(bi), widen(bo)
    oi = oo = 0
    errs, ulps = [], []
    for xin, xout, meta, first, alpha in batches:
        dIn, dOut = oracle_mod.minibatch(xin, xout, meta, first, float(alpha), acc64=True)
        I, O = xin.shape[0], xout.shape[0]
        for stored, base, upd in ((ri[oi:oi + I], xin, dIn), (ro[oo:oo + O], xout, dOut)):
            new64 = base.astype(np.float64) + upd
            errs.append(np.max(np.linalg.norm(stored - new64, axis=1) / np.maximum(np.linalg.norm(new64, axis=1), 1e-30)))
            nz = new64 != 0
            ulps.append(np.mean((stored[nz] - new64[nz]) / 2.0 ** (np.floor(np.log2(np.abs(new64[nz]))) - 7)))
        oi += I
        oo += O
    errs = np.array(errs)
    assert errs.max() <= 2.0 ** -7 * 1.001, errs.max()
    assert np.median(errs) < 4e-3, np.median(errs)
    assert abs(np.mean(ulps)) < 0.02, np.mean(ulps)
