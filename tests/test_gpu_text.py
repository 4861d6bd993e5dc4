"""GPU rating-text converter (data/netflix/transform.cpp) against the reference's own
transform output (golden fixtures) and the oracle's strict parse on large random texts."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu


def fixtures():
    z = np.load(os.path.join(GOLDEN, "text.npz"))
    return {k[5:]: (z[k].tobytes(), z["bin_" + k[5:]].tobytes()) for k in z.files if k.startswith("text_")}


def test_convert_matches_reference_transform(lib, cuda, tmp_path):
    import cumf_sgd_gb300 as cm
    for name, (text, ref) in fixtures().items():
        src = tmp_path / name
        src.write_bytes(text)
        n = cm.convert_text(str(src))
        assert n * 12 == len(ref), name
        assert (tmp_path / (name + ".bin")).read_bytes() == ref, name


def test_transform_tool_writes_reference_records(lib, cuda, tmp_path):
    text, ref = fixtures()["decimals"]
    src = tmp_path / "netflix_train"
    src.write_bytes(text)
    exe = os.path.join(ROOT, "cumf_sgd_gb300", "bin", "cumf_transform")
    res = subprocess.run([exe, str(src)], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout
    assert (tmp_path / "netflix_train.bin").read_bytes() == ref


def random_text(n, seed):
    rng = np.random.default_rng(seed)
    u = rng.integers(0, 2_000_000, n)
    v = rng.integers(0, 20_000, n)
    kind = rng.integers(0, 6, n)
    r = np.where(kind == 0, rng.integers(1, 6, n).astype(np.float64),
                 np.where(kind < 3, rng.uniform(0, 5, n), 10.0 ** rng.uniform(-44, 38, n)))
    fmts = ["%d", "%.1f", "%.9g", "%.17g", "%.6e", "%.18e"]
    seps = [" ", "\t", "  "]
    ends = ["\n", "\r\n", " \n"]
    out = ["%%%%MatrixMarket matrix coordinate real general\n%%\n2000000 20000 %d\n" % n]
    for i in range(n):
        f = fmts[kind[i]]
        rv = ("%d" % r[i]) if f == "%d" else (f % r[i])
        out.append("%d%s%d%s%s%s" % (u[i], seps[i % 3], v[i], seps[(i + 1) % 3], rv, ends[i % 3]))
    return "".join(out).encode()


@pytest.mark.parametrize("n,seed", [(1, 1), (1000, 2), (300_000, 3)])
def test_device_parse_matches_oracle(lib, cuda, orc, n, seed):
    import torch
    import cumf_sgd_gb300 as cm
    text = random_text(n, seed)
    exp = orc.parse_text(text)
    assert len(exp) == n
    d = torch.frombuffer(bytearray(text + b"\0" * 16), dtype=torch.uint8).to(cuda)
    start = cm.text_data_start(text)
    cnt = cm.dev_parse_text(d.data_ptr(), len(text), start)
    assert cnt == n
    out = torch.empty(n * 12, dtype=torch.uint8, device=cuda)
    assert cm.dev_parse_text(d.data_ptr(), len(text), start, out.data_ptr(), n) == n
    got = out.cpu().numpy().tobytes()
    assert got == exp.tobytes()


def test_read_text_problem_extent(lib, cuda, tmp_path):
    import cumf_sgd_gb300 as cm
    text = b"a\nb\nc\n3 7 1.5\n0 2 4\n12 0 2.25\n"
    p = tmp_path / "t.txt"
    p.write_bytes(text)
    prob = cm.read_text_problem(str(p))
    assert (prob.m, prob.n, prob.nnz) == (13, 8, 3)
    assert list(prob.records["r"]) == [1.5, 4.0, 2.25]
    p.write_bytes(b"a\nb\nc\n-3 7 1.5\n")
    with pytest.raises(cm.CumfError):
        cm.read_text_problem(str(p))


@pytest.mark.parametrize("body,where", [
    (b"1 2 3\n4 5 x\n", 10), (b"1 2.5 3\n", 2), (b"1 2 0x1p3\n", 4), (b"99999999999 2 3\n", 0),
    (b"1 2 3.5.5\n", 4), (b"1 2 1e\n", 4), (b"1 2 --3\n", 4), (b"1 2 nan(1)\n", 4), (b"1 +-2 3\n", 2)])
def test_malformed_tokens_fail_at_the_oracle_offset(lib, cuda, orc, tmp_path, body, where):
    import cumf_sgd_gb300 as cm
    from cumf_sgd_gb300 import _lib
    head = b"a\nb\nc\n"
    assert orc.parse_text(head + body) == ("bad", len(head) + where)
    p = tmp_path / "bad.txt"
    p.write_bytes(head + body)
    with pytest.raises(cm.CumfError) as e:
        cm.convert_text(str(p))
    assert e.value.code == _lib.CUMF_ERR_FORMAT
    assert "byte %d:" % (len(head) + where) in str(e.value)


def test_partial_triple_and_long_digits(lib, cuda, orc, tmp_path):
    import cumf_sgd_gb300 as cm
    from cumf_sgd_gb300 import _lib
    p = tmp_path / "t.txt"
    p.write_bytes(b"a\nb\nc\n1 2 3 4\n")
    with pytest.raises(cm.CumfError) as e:
        cm.convert_text(str(p))
    assert e.value.code == _lib.CUMF_ERR_FORMAT
    # More than 19 significant digits: accepted when the dropped digits cannot change the
    # rounding, rejected when they could (strtof would resolve it with all the digits).
    p.write_bytes(b"a\nb\nc\n1 2 1.00000000000000000000001\n")
    assert cm.convert_text(str(p)) == 1
    ref = orc.parse_text(p.read_bytes())
    assert (tmp_path / "t.txt.bin").read_bytes() == ref.tobytes()
    p.write_bytes(b"a\nb\nc\n1 2 1.0000000596046447753906250000001\n")
    with pytest.raises(cm.CumfError) as e:
        cm.convert_text(str(p))
    assert "19 significant digits" in str(e.value)


def test_capacity_errors(lib, cuda):
    import torch
    import cumf_sgd_gb300 as cm
    text = b"1 2 3\n4 5 6\n"
    d = torch.frombuffer(bytearray(text + b"\0" * 16), dtype=torch.uint8).to(cuda)
    out = torch.empty(12, dtype=torch.uint8, device=cuda)
    with pytest.raises(cm.CumfError):
        cm.dev_parse_text(d.data_ptr(), len(text), 0, out.data_ptr(), 1)
    with pytest.raises(cm.CumfError):  # misaligned text
        cm.dev_parse_text(d.data_ptr() + 1, len(text) - 1, 0)


@pytest.mark.parametrize("body,where", [
    (b"1 2 .e5\n", 4), (b"1 2 1e+\n", 4), (b"1 2 -\n", 4), (b"1 2 +.\n", 4), (b"1 2 1.5e5.5\n", 4),
    (b"12a 2 3\n", 0), (b"1 - 3\n", 2), (b"1 2 e5\n", 4), (b"1 2 1..\n", 4), (b"3000000000 2 3\n", 0)])
def test_malformed_short_tokens_mid_text(lib, cuda, orc, tmp_path, body, where):
    """Short malformed tokens followed by more text: rejected at the oracle's offset."""
    import cumf_sgd_gb300 as cm
    from cumf_sgd_gb300 import _lib
    head = b"a\nb\nc\n"
    text = head + body + b"7 8 9\n" * 12
    assert orc.parse_text(text) == ("bad", len(head) + where)
    p = tmp_path / "bad.txt"
    p.write_bytes(text)
    with pytest.raises(cm.CumfError) as e:
        cm.convert_text(str(p))
    assert e.value.code == _lib.CUMF_ERR_FORMAT
    assert "byte %d:" % (len(head) + where) in str(e.value)


def test_valid_spellings_mid_text(lib, cuda, orc, tmp_path):
    import cumf_sgd_gb300 as cm
    toks = [b"+4", b"007", b"-0.0", b"4.", b".5", b"-.25", b"1e-3", b"2.5E+1", b"5e0", b"0e10", b"16777217",
            b"0.1", b"3.4e38", b"1e-45", b"inf", b"-nan", b"123456789012345", b"1.25e-07"]
    body = b"".join(b"%d %d %s\n" % (i, i + 1, t) for i, t in enumerate(toks)) + b"7 8 9\n" * 12
    text = b"a\nb\nc\n" + body
    p = tmp_path / "ok.txt"
    p.write_bytes(text)
    assert cm.convert_text(str(p)) == len(toks) + 12
    assert (tmp_path / "ok.txt.bin").read_bytes() == orc.parse_text(text).tobytes()


def test_host_pipeline_matches_oracle_across_chunks(lib, cuda, orc):
    """More than one 64 MB chunk: records that straddle chunk boundaries, copies overlapped."""
    import cumf_sgd_gb300 as cm
    block = random_text(200_000, 11)
    head_end = cm.text_data_start(block)
    body = block[head_end:]
    text = block[:head_end] + body * ((70 << 20) // len(body) + 1)
    exp = orc.parse_text(text)
    got = cm.parse_text_host(text)
    assert len(got) == len(exp) and got.tobytes() == exp.tobytes()
    for name, (small, ref) in fixtures().items():
        assert cm.parse_text_host(small).tobytes() == ref, name


EDGE_IDS = [b"0", b"7", b"007", b"123456", b"1234567", b"12345678", b"2147483647", b"0000000000012", b"+5"]
EDGE_RATINGS = [b"4", b"3.5", b".5", b"5.", b"0", b"0.0", b"007.25", b"1234567", b"12345.6", b"9999999",
                b"0.000001", b"1e3", b"+2", b"-1.5", b"inf", b"1.23456789", b"3.14159", b"0.1", b".000001",
                b"16777217", b"9.99999", b"-0", b"2.5E+1"]


def edge_text(n, seed, tail_newline=True):
    """Records of edge spellings with ragged separators, so that tokens of every length start
    at every offset of the 64-byte segments and of the 16 KB blocks (and in the halo)."""
    rng = np.random.default_rng(seed)
    seps = [b" ", b"\t", b"  ", b"\x0b", b"\x0c", b" \r"]
    out = [b"h1\nh2\nh3\n"]
    for i in range(n):
        u = EDGE_IDS[rng.integers(len(EDGE_IDS))]
        v = EDGE_IDS[rng.integers(len(EDGE_IDS))]
        r = EDGE_RATINGS[rng.integers(len(EDGE_RATINGS))]
        pad = b" " * int(rng.integers(0, 3))
        out.append(pad + u + seps[rng.integers(len(seps))] + v + seps[rng.integers(len(seps))] + r + b"\n")
    text = b"".join(out)
    return text if tail_newline else text.rstrip(b"\n")


@pytest.mark.parametrize("n,seed,tail", [(40_000, 21, True), (40_000, 22, False), (3, 23, False), (1500, 24, True)])
def test_edge_spellings_match_oracle(lib, cuda, orc, n, seed, tail):
    """Short tokens (byte-parallel path) and long, signed or exponent tokens (general path)
    mixed, across segment, block and halo boundaries; text ending with and without a newline."""
    import torch
    import cumf_sgd_gb300 as cm
    text = edge_text(n, seed, tail)
    exp = orc.parse_text(text)
    assert len(exp) == n
    start = cm.text_data_start(text)
    d = torch.frombuffer(bytearray(text + b"\0" * 16), dtype=torch.uint8).to(cuda)
    out = torch.empty(n * 12, dtype=torch.uint8, device=cuda)
    assert cm.dev_parse_text(d.data_ptr(), len(text), start, out.data_ptr(), n) == n
    assert out.cpu().numpy().tobytes() == exp.tobytes()
    assert cm.parse_text_host(text).tobytes() == exp.tobytes()


@pytest.mark.parametrize("bad", [b"4\x01", b"4\x80", b"\x7f", b"4..5", b"3.5.", b"..", b"1\x1f2", b"9\xff"])
@pytest.mark.parametrize("where", [0, 1, 2])
def test_short_malformed_tokens_at_the_oracle_offset(lib, cuda, orc, tmp_path, bad, where):
    """Short tokens with control, high or repeated '.' bytes are refused by the byte-parallel
    path and rejected by the general parser at the oracle's offset (field `where`)."""
    import cumf_sgd_gb300 as cm
    from cumf_sgd_gb300 import _lib
    fields = [b"11", b"22", b"3.5"]
    fields[where] = bad
    text = b"a\nb\nc\n" + b"7 8 9\n" * 5000 + b" ".join(fields) + b"\n" + b"7 8 9\n" * 5
    exp = orc.parse_text(text)
    assert exp[0] == "bad"
    p = tmp_path / "bad.txt"
    p.write_bytes(text)
    with pytest.raises(cm.CumfError) as e:
        cm.convert_text(str(p))
    assert e.value.code == _lib.CUMF_ERR_FORMAT
    assert "byte %d:" % exp[1] in str(e.value)
