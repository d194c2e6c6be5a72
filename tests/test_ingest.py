"""Walk-file text -> corpus: the GPU parser (sgns_parse_walks, sgns_train_walk_files)
against the oracle's restatement of the reference reader (word2vec.cu:1002-1041 on the
format of path.hpp:92,108)."""
import os

import numpy as np
import pytest

import sgns

EDGE_CASES = [
    (b" 1 2 3\n 4 5\n", 0, [1, 2, 3, -1, 4, 5, -1]),
    (b"1 2", 0, [1, 2, -1]),                       # no final newline: the end closes the walk
    (b"\n\n 7\r\n\t8 \n", 0, [7, -1, 8, -1]),      # empty lines, CRLF, tab
    (b"", 0, []),
    (b"   \n\t\r\n", 0, []),
    (b" 2147483647\n", 0, [2147483647, -1]),
    (b" 0000000007\n", 0, [7, -1]),               # ten digits with leading zeros
    (b" 00000000007\n", 2, None),                 # eleven digits
    (b" 2147483648\n", 2, None),
    (b" 1 x 2\n", 1, None),
    (b" 3\n\n\n 4", 0, [3, -1, 4, -1]),
]


def python_parse(text):
    """The reader's rules as a plain loop (small inputs only)."""
    if any(c not in b"0123456789 \t\r\n" for c in text):
        return 1, None
    out, cur, line = [], None, False
    for c in text + b"\n":
        if 48 <= c <= 57:
            cur = (cur or "") + chr(c)
            continue
        if cur is not None:
            if len(cur) > 10 or int(cur) > 2147483647:
                return 2, None
            out.append(int(cur))
            line, cur = True, None
        if c == 10:
            if line:
                out.append(-1)
            line = False
    return 0, out


def random_text(rng, n_lines, with_noise=True):
    parts = []
    for _ in range(n_lines):
        k = int(rng.integers(0, 12))
        ids = rng.integers(0, 2**31 - 1 if rng.random() < 0.1 else 5000, size=k)
        line = []
        for v in ids:
            sep = rng.choice([b" ", b"\t", b"  ", b" " * int(rng.integers(1, 80))]) if with_noise else b" "
            s = str(int(v)).encode()
            if with_noise and rng.random() < 0.05:
                s = b"0" * int(rng.integers(1, 10 - len(s) + 1)) + s if len(s) < 10 else s
            line.append(sep + s)
        end = rng.choice([b"\n", b"\r\n", b" \n", b"\n\n"]) if with_noise else b"\n"
        parts.append(b"".join(line) + end)
    text = b"".join(parts)
    if with_noise and rng.random() < 0.5:
        text = text.rstrip(b"\n")
    return text


@pytest.mark.parametrize("text,code,tokens", EDGE_CASES)
def test_oracle_parse_edge_cases(text, code, tokens, oracle_mod):
    c, out, mx, err = oracle_mod.parse_walks(text)
    assert c == code
    if code == 0:
        assert out.tolist() == tokens
        assert mx == (max([t for t in tokens if t >= 0]) if any(t >= 0 for t in tokens) else -1)


def test_oracle_parse_matches_the_rules_on_random_text(oracle_mod):
    rng = np.random.default_rng(5)
    for _ in range(40):
        text = random_text(rng, int(rng.integers(0, 30)))
        code, ref = python_parse(text)
        c, out, _, _ = oracle_mod.parse_walks(text)
        assert c == code
        if code == 0:
            assert out.tolist() == ref


def _gpu_parse(text, torch):
    t = torch.tensor(np.frombuffer(text, np.uint8).copy(), device="cuda") if text else torch.empty(0, dtype=torch.uint8, device="cuda")
    n = sgns.parse_walks_count(t)
    tok = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    n2, mx = sgns.parse_walks(t, tok)
    torch.cuda.synchronize()
    return tok[:n2].cpu().numpy(), mx


@pytest.mark.gpu
def test_gpu_parse_matches_oracle(sgns_lib, oracle_mod):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    texts = [t for t, c, _ in EDGE_CASES if c == 0]
    texts += [random_text(rng, n) for n in (1, 3, 200, 1200, 9000, 60000)]
    # blank runs longer than a thread's 32 bytes and than an 8 KB tile
    texts.append(b" 5" + b" " * 40 + b"\n" + b" " * 20000 + b"\n 6 7" + b"\t" * 9000 + b" 8\n")
    texts.append(b"\n" * 10000 + b" 123" + b" " * 8190 + b"\n")
    # ids cut by tile edges: ids of every length ending at offsets around 8192
    for shift in range(0, 12):
        texts.append(b" " * (8192 - shift) + b"1234567890 42\n 9")
    for text in texts:
        c, ref, mx, _ = oracle_mod.parse_walks(text)
        assert c == 0
        out, gmx = _gpu_parse(text, torch)
        assert np.array_equal(out, ref), (len(text), len(out), len(ref))
        assert gmx == mx
    # text that does not start on a 16-byte boundary (a view at an odd offset)
    text = random_text(rng, 3000)
    _, ref, mx, _ = oracle_mod.parse_walks(text)
    buf = torch.tensor(np.frombuffer(b"123" + text, np.uint8).copy(), device="cuda")
    view = buf[3:]
    assert view.data_ptr() % 16 != 0
    tok = torch.empty(len(ref), dtype=torch.int32, device="cuda")
    assert sgns.parse_walks(view, tok) == (len(ref), mx)
    assert np.array_equal(tok.cpu().numpy(), ref)


@pytest.mark.gpu
def test_gpu_parse_across_scan_groups(sgns_lib, oracle_mod):
    """Texts longer than one scan group (1024 tiles of 8 KB), so the tile prefixes come from
    the two-level scan: ordinary walks over several groups, whole groups of blanks or
    newlines, a walk that spans them and ids cut by a group edge."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    block = random_text(rng, 20000) + b"\n"
    group = 1024 * 8192
    texts = [block * 7,
             block + b" " * (group + 100) + b" 77 78" + b" " * group + b"\n 79\n" + block,
             b"\n" * (2 * group + 5) + b" 1 2 3"]
    for shift in (0, 1, 5):
        texts.append(b" " * (group - shift) + b"1234567 42\n 9")
    for text in texts:
        c, ref, mx, _ = oracle_mod.parse_walks(text)
        assert c == 0
        out, gmx = _gpu_parse(text, torch)
        assert np.array_equal(out, ref), (len(text), len(out), len(ref))
        assert gmx == mx


@pytest.mark.gpu
def test_gpu_parse_errors(sgns_lib, oracle_mod):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(12)
    base = random_text(rng, 3000, with_noise=False)
    cases = []
    for off in (0, 1, 8191, 8192, len(base) // 2, len(base) - 1):
        b = bytearray(base)
        b[off] = ord("x")
        cases.append(bytes(b))
    cases.append(base + b" 99999999999\n")
    cases.append(base[:5000] + b" 2147483648 " + base[5000:])
    for text in cases:
        c, _, _, err = oracle_mod.parse_walks(text)
        assert c in (1, 2)
        t = torch.tensor(np.frombuffer(text, np.uint8).copy(), device="cuda")
        with pytest.raises(sgns.SgnsError) as e:
            n = sgns.parse_walks_count(t)
            tok = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
            sgns.parse_walks(t, tok)
        assert e.value.status == sgns.EINVAL and ("offset %d " % err) in str(e.value)
    # too small a capacity reports the count and writes nothing
    t = torch.tensor(np.frombuffer(base, np.uint8).copy(), device="cuda")
    n = sgns.parse_walks_count(t)
    tok = torch.full((n - 1,), -7, dtype=torch.int32, device="cuda")
    with pytest.raises(sgns.SgnsError):
        sgns.parse_walks(t, tok)
    assert bool((tok == -7).all())


@pytest.mark.gpu
def test_train_walk_files_equals_training_on_the_parsed_corpus(sgns_lib, oracle_mod, tmp_path):
    """Files written in the reference's format (one of them with CRLF and no final
    newline) give the same model as training on the oracle-parsed corpus."""
    import synth

    ip, ix = synth.chung_lu(3000, 20000, 2.1, seed=41)
    c = synth.random_walks(ip, ix, 2, 30, seed=42).numpy().astype(np.int32)
    ends = np.flatnonzero(c == -1)
    half = ends[len(ends) // 2] + 1
    p1, p2 = str(tmp_path / "w0.txt"), str(tmp_path / "w1.txt")
    synth.write_walk_file(c[:half], p1)
    synth.write_walk_file(c[half:], p2)
    raw = open(p2, "rb").read().replace(b"\n", b"\r\n").rstrip(b"\r\n")
    open(p2, "wb").write(raw)
    texts = open(p1, "rb").read() + b"\n" + raw + b"\n"
    code, parsed, mx, _ = oracle_mod.parse_walks(texts)
    assert code == 0 and np.array_equal(parsed, c)
    opt = dict(size=64, window=5, negative=5, iter=1, sample=1e-3, alpha=0.025, table_size=1000000, debug=0,
               engine="plain", mode="exact")
    with sgns.Trainer(**opt) as t:
        st = t.train_walk_files([p1, p2])
        w1, o1 = t.embeddings(0), t.order()
    with sgns.Trainer(**opt) as t:
        t.set_vocab(np.bincount(parsed[parsed >= 0], minlength=mx + 1).astype(np.int32))
        st2 = t.train_corpus(parsed)
        w2, o2 = t.embeddings(0), t.order()
    assert (st.steps, st.pairs, st.word_count_actual) == (st2.steps, st2.pairs, st2.word_count_actual)
    assert np.array_equal(o1, o2) and np.array_equal(w1.view(np.uint32), w2.view(np.uint32))
