"""CONTRAfold binary output formats (parens, sparse posteriors): written here,
read back the way the reference reads the binary's files
(gpu_contrafold/reference.py:61-132), on the golden posterior matrices."""
import io

import numpy as np
import pytest

from conftest import golden_post
from contrafold_gpu_gb300 import formats


def _bpp(rec):
    L = len(rec["seq"])
    return golden_post(rec)[1:L + 1, 1:L + 1].astype(np.float64)


def test_posteriors_round_trip_golden(tmp_path, golden):
    cases = [c for c in golden["cases"] if 0 < len(c["seq"]) <= 120][:12]
    assert cases
    for k, c in enumerate(cases):
        seq, mat = c["seq"], _bpp(c)
        for cutoff in (0.0, 1e-5, 0.01, 0.5):
            path = tmp_path / f"p{k}.post"
            formats.write_posteriors_file(str(path), [(f"s{k}", seq, mat)], cutoff)
            back = formats.read_posteriors(str(path), len(seq))
            upper = np.triu(mat, 1)
            keep = upper >= cutoff
            # six significant digits; entries below the cutoff are not listed
            assert np.allclose(back[keep], upper[keep], rtol=5e-6, atol=0)
            assert np.all(back[~keep] == 0)
            assert np.all(np.tril(back) == 0)


def test_posteriors_layout():
    fh = io.StringIO()
    mat = np.zeros((4, 4))
    mat[0, 3] = 0.25
    mat[1, 2] = 1e-7
    formats.write_posteriors(fh, "GACU", mat, cutoff=1e-5)
    assert fh.getvalue().splitlines() == ["1 G 4:0.25", "2 A", "3 C", "4 U"]
    fh = io.StringIO()
    formats.write_posteriors(fh, "GACU", mat, cutoff=0.0, name="x")
    assert fh.getvalue().splitlines()[:3] == [">x", "1 G 2:0 3:0 4:0.25", "2 A 3:1e-07 4:0"]
    with pytest.raises(ValueError):
        formats.write_posteriors(io.StringIO(), "GAC", mat)


def test_posteriors_reader_takes_either_order(tmp_path):
    p = tmp_path / "x.post"
    p.write_text(">s\n1 G 4:0.5\n4 C 2:0.125\n")
    m = formats.read_posteriors(str(p), 4)
    assert m[0, 3] == 0.5 and m[1, 3] == 0.125 and m.sum() == 0.625


def test_parens(tmp_path, golden):
    c = next(c for c in golden["cases"] if len(c["seq"]) > 10)
    p = tmp_path / "a.parens"
    formats.write_parens_file(str(p), [("r", c["seq"], c["mea"]["6.0"])])
    assert p.read_text() == f">r\n{c['seq']}\n{c['mea']['6.0']}\n"
    assert formats.read_parens(str(p)) == c["mea"]["6.0"]
    with pytest.raises(ValueError):
        formats.write_parens(io.StringIO(), "r", "ACGU", "(.)")
