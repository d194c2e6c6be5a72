"""sgns_minibatch_update_noalloc, the entry point for callers that cannot let the
library allocate device memory (their GPU memory is owned by their own allocator).

It must give the same rows as sgns_minibatch_update -- bit for bit, the tolerance of the
other minibatch tests -- on consecutive calls (its static scratch keeps the previous
call's contents, including the status word that has to start at zero), and reject a
batch count beyond its static limit.  Collected last so a run that stops at the first
failure has run every other test already; it also passes alone in a fresh process."""
import numpy as np
import pytest

import sgns

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def batches(n, d, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        I = int(rng.integers(2, 41))
        first = int(rng.integers(1, I))
        O = int(rng.integers(2, 13))
        meta = np.ones(O, np.int32)
        meta[1:O - 1] = rng.integers(1, 4, O - 2)
        xin = (rng.standard_normal((I, d)) * 0.3 / np.sqrt(d)).astype(np.float32)
        xout = (rng.standard_normal((O, d)) * 0.3).astype(np.float32)
        out.append((xin, xout, meta, first, np.float32(rng.uniform(1e-4, 0.05))))
    return out


def device_args(bs):
    dev = "cuda"
    a = dict(
        in_count=torch.tensor([b[0].shape[0] for b in bs], dtype=torch.int32, device=dev),
        in_first=torch.tensor([b[3] for b in bs], dtype=torch.int32, device=dev),
        out_count=torch.tensor([b[1].shape[0] for b in bs], dtype=torch.int32, device=dev),
        out_meta=torch.tensor(np.concatenate([b[2] for b in bs]), device=dev),
        alpha=torch.tensor([b[4] for b in bs], dtype=torch.float32, device=dev),
        in_rows=torch.tensor(np.concatenate([b[0] for b in bs]), device=dev),
        out_rows=torch.tensor(np.concatenate([b[1] for b in bs]), device=dev),
    )
    return a


def run(fn, d, a):
    d_in = torch.full_like(a["in_rows"], float("nan"))
    d_out = torch.full_like(a["out_rows"], float("nan"))
    fn(d, a["in_count"], a["in_first"], a["out_count"], a["out_meta"], a["alpha"], a["in_rows"], a["out_rows"],
       d_in, d_out, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return d_in.cpu().numpy(), d_out.cpu().numpy()


@pytest.mark.parametrize("d", [128, 64])
def test_noalloc_matches_allocating_entry_point_on_consecutive_calls(d):
    for call, seed in enumerate((11 + d, 12 + d)):  # two calls in a row, different shapes
        a = device_args(batches(300 + 17 * call, d, seed))
        ref_in, ref_out = run(sgns.minibatch_update, d, a)
        got_in, got_out = run(sgns.minibatch_update_noalloc, d, a)
        assert np.array_equal(got_in.view(np.uint32), ref_in.view(np.uint32)), call
        assert np.array_equal(got_out.view(np.uint32), ref_out.view(np.uint32)), call


def test_noalloc_status_is_cleared_between_calls():
    d = 32
    bad = batches(4, d, 3)
    x = bad[1]
    bad[1] = (np.zeros((70, d), np.float32), x[1], x[2], 1, x[4])  # 70 inputs: over the limit
    with pytest.raises(sgns.SgnsError) as e:
        run(sgns.minibatch_update_noalloc, d, device_args(bad))
    assert e.value.status == sgns.EINVAL
    a = device_args(batches(8, d, 4))  # the next call must not see the stale status
    ref_in, ref_out = run(sgns.minibatch_update, d, a)
    got_in, got_out = run(sgns.minibatch_update_noalloc, d, a)
    assert np.array_equal(got_in, ref_in) and np.array_equal(got_out, ref_out)


def test_noalloc_rejects_more_batches_than_its_scratch_holds():
    d = 16
    n = 65537
    dev = "cuda"
    ones = torch.full((n,), 2, dtype=torch.int32, device=dev)
    with pytest.raises(sgns.SgnsError) as e:
        sgns.minibatch_update_noalloc(d, ones, torch.ones(n, dtype=torch.int32, device=dev), ones,
                                      torch.ones(2 * n, dtype=torch.int32, device=dev),
                                      torch.zeros(n, device=dev), torch.zeros((2 * n, d), device=dev),
                                      torch.zeros((2 * n, d), device=dev), torch.zeros((2 * n, d), device=dev),
                                      torch.zeros((2 * n, d), device=dev))
    assert e.value.status == sgns.EINVAL
    assert "65536" in str(e.value)
