"""CLI: input sniffing and mask validation (CPU), end-to-end JSONL runs (GPU)."""
import json
import subprocess
import sys

import numpy as np
import pytest

from contrafold_gpu_gb300 import cli


def test_load_records_formats(tmp_path):
    j = tmp_path / "a.jsonl"
    j.write_text('{"id": "r1", "seq": "ggggaaaacccc", "constrain": "000100000000"}\n\n{"seq": "ACGU"}\n')
    recs, from_file = cli.load_records(str(j))
    assert from_file and recs == [("r1", "GGGGAAAACCCC", "000100000000"), (2, "ACGU", None)]
    f = tmp_path / "a.fa"
    f.write_text(">x\nGGGG\nAAAA\n>\nCCCC\n")
    assert cli.load_records(str(f))[0] == [("x", "GGGGAAAA", None), (1, "CCCC", None)]
    t = tmp_path / "a.txt"
    t.write_text("acgu\n\nGGCC\n")
    assert cli.load_records(str(t))[0] == [(0, "ACGU", None), (2, "GGCC", None)]
    assert cli.load_records("acgun") == ([(0, "ACGUN", None)], False)
    with pytest.raises(SystemExit):
        cli.load_records("not-a-sequence!")


def test_jsonl_errors(tmp_path):
    bad = tmp_path / "b.jsonl"
    bad.write_text('{"id": 1}\n')
    with pytest.raises(SystemExit, match="missing required field"):
        cli.load_records(str(bad))
    bad.write_text('{"seq": \n')
    with pytest.raises(SystemExit, match="invalid JSON"):
        cli.load_records(str(bad))


def test_input_behaviour_edges(tmp_path):
    """A FASTA record without sequence is dropped (and does not count for the
    next unnamed header); a JSON line that is not an object has no 'seq';
    leading blank lines do not decide the format; any character but '1' in a
    constrain string is 0."""
    f = tmp_path / "e.fa"
    f.write_text("\n\n>empty\n>\nGG CC \n\n>z\nau\n")
    assert cli.load_records(str(f))[0] == [(0, "GG CC", None), ("z", "AU", None)]
    j = tmp_path / "e.jsonl"
    j.write_text('\n{"seq": "GGGAAACCC", "id": 7}\n[1, 2]\n')
    with pytest.raises(SystemExit, match="line 2: missing required field"):
        cli.load_records(str(j))
    assert cli.build_mask("ACGU", "01x1").tolist() == [0, 1, 0, 1]
    assert cli.build_mask("ACGU", "") is None and cli.build_mask("ACGU", []) is None
    with pytest.raises(SystemExit):
        cli.load_records("ACGX")


def test_build_mask():
    assert cli.build_mask("ACGU", None) is None
    assert cli.build_mask("ACGU", "0101").tolist() == [0, 1, 0, 1]
    assert cli.build_mask("ACGU", [1, 0, 0, 1]).dtype == np.int8
    with pytest.raises(SystemExit, match="length"):
        cli.build_mask("ACGU", "01")
    with pytest.raises(SystemExit, match="expected 0 or 1"):
        cli.build_mask("ACGU", [0, 2, 0, 0])


def _run(args, cwd):
    return subprocess.run([sys.executable, "-m", "contrafold_gpu_gb300", *args], capture_output=True, text=True,
                          cwd=cwd)


@pytest.mark.gpu
def test_cli_end_to_end(tmp_path, P, oracle, golden):
    import os
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = _run(["GGGGAAAACCCC"], repo)
    assert r.returncode == 0 and r.stdout.strip() == "((((....))))", r.stderr
    r = _run(["GGGGAAAACCCC", "--viterbi"], repo)
    assert r.stdout.strip() == "((((....))))"
    r = _run(["GGGGAAAACCCC", "--logz"], repo)
    assert abs(float(r.stdout) - 3.05661) < 5e-4
    r = _run(["GGGGAAAACCCC", "--sample", "5", "--logz", "--seed", "3"], repo)
    lines = r.stdout.strip().splitlines()
    assert lines[0].startswith("# logZ = ") and len(lines) == 6
    recs = [c for c in golden["cases"] if 8 <= len(c["seq"]) <= 60][:30]
    src = tmp_path / "in.jsonl"
    with open(src, "w") as fh:
        for k, c in enumerate(recs):
            obj = {"id": f"s{k}", "seq": c["seq"]}
            if c["mask"]:
                obj["constrain"] = c["mask"]
            fh.write(json.dumps(obj) + "\n")
    out = tmp_path / "out.jsonl"
    r = _run([str(src), "-o", str(out), "--chunk", "7"], repo)
    assert r.returncode == 0, r.stderr
    got = [json.loads(l) for l in open(out)]
    assert [g["id"] for g in got] == [f"s{k}" for k in range(len(recs))]
    assert [g["structure"] for g in got] == [c["mea"]["6.0"] for c in recs]
    r = _run([str(src), "-o", str(out), "--viterbi"], repo)
    assert [json.loads(l)["structure"] for l in open(out)] == [c["mfe"] for c in recs]


@pytest.mark.gpu
def test_cli_contrafold_files(tmp_path, golden):
    """--parens / --posteriors: the binary's file formats, read back as the
    reference reads them, equal the golden MEA structures and posteriors."""
    import os

    from conftest import golden_post
    from contrafold_gpu_gb300 import formats
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    recs = [c for c in golden["cases"] if 8 <= len(c["seq"]) <= 80][:10]
    src = tmp_path / "in.jsonl"
    with open(src, "w") as fh:
        for k, c in enumerate(recs):
            obj = {"id": f"s{k}", "seq": c["seq"]}
            if c["mask"]:
                obj["constrain"] = c["mask"]
            fh.write(json.dumps(obj) + "\n")
    par, post, out = tmp_path / "o.parens", tmp_path / "o.post", tmp_path / "o.jsonl"
    r = _run([str(src), "-o", str(out), "--parens", str(par), "--posteriors", "1e-4", str(post)], repo)
    assert r.returncode == 0, r.stderr
    lines = par.read_text().splitlines()
    assert len(lines) == 3 * len(recs)
    for k, c in enumerate(recs):
        assert lines[3 * k:3 * k + 3] == [f">s{k}", c["seq"].upper(), c["mea"]["6.0"]]
    blocks, cur = [], None
    for line in post.read_text().splitlines():
        if line.startswith(">"):
            cur = []
            blocks.append(cur)
        else:
            cur.append(line)
    assert len(blocks) == len(recs)
    for k, c in enumerate(recs):
        L = len(c["seq"])
        one = tmp_path / f"one{k}.post"
        one.write_text("\n".join(blocks[k]) + "\n")
        got = formats.read_posteriors(str(one), L)
        want = np.triu(golden_post(c)[1:L + 1, 1:L + 1].astype(np.float64), 1)
        keep = want >= 1e-4
        assert np.allclose(got[keep], want[keep], rtol=5e-6, atol=0) and np.all(got[~keep] == 0)
    r = _run(["GGGGAAAACCCC", "--logz", "--parens", str(par)], repo)
    assert r.returncode != 0 and "--parens" in r.stderr


def test_contrafold_file_options_validated_before_folding(tmp_path):
    """--parens needs a structure mode and --posteriors a numeric cutoff; both are
    rejected before any sequence is folded (no GPU needed)."""
    with pytest.raises(SystemExit, match="--parens"):
        cli.main(["GGGGAAAACCCC", "--logz", "--parens", str(tmp_path / "a.parens")])
    with pytest.raises(SystemExit, match="--parens"):
        cli.main(["GGGGAAAACCCC", "--sample", "3", "--parens", str(tmp_path / "a.parens")])
    with pytest.raises(SystemExit, match="not a number"):
        cli.main(["GGGGAAAACCCC", "--posteriors", "abc", str(tmp_path / "a.post")])
    assert not (tmp_path / "a.parens").exists() and not (tmp_path / "a.post").exists()
