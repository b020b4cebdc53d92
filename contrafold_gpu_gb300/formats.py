"""Output files in the formats of the CONTRAfold binary's `predict` command, as
the reference reads them back (gpu_contrafold/reference.py:61-132):

* parens (`predict --parens FILE`): per record a `>name` line, the sequence
  and the dot-bracket structure; the reference takes the last line
  (reference.py:70-74, 93-95).
* posteriors (`predict --posteriors CUTOFF FILE`): one line per position i
  (1-based), `i base j:p j:p ...`, listing the partners j with P(i, j) >= CUTOFF;
  the reader fills the upper triangle from either order of (i, j)
  (reference.py:112-125).  Lines of fewer than two fields are skipped by that
  reader, so the `>name` line written before each record's block (files with
  several records) is harmless to it.

The binary itself is not part of the reference, so these follow the formats
as the reference parses them; probabilities are written with six significant
digits (an ostream's default precision).
"""
from __future__ import annotations

from typing import IO, Iterable, Optional, Tuple

import numpy as np


def write_parens(fh: IO[str], name, seq: str, structure: str) -> None:
    """One record of a parens file: `>name`, sequence, structure."""
    if len(structure) != len(seq):
        raise ValueError("structure and sequence lengths differ")
    fh.write(f">{name}\n{seq}\n{structure}\n")


def read_parens(path: str) -> str:
    """The structure of a single-record parens file: its last line
    (reference.py:70-74)."""
    with open(path) as fh:
        lines = [ln.rstrip("\n") for ln in fh]
    return lines[-1].strip()


def write_posteriors(fh: IO[str], seq: str, bpp: np.ndarray, cutoff: float = 1e-5,
                     name: Optional[object] = None) -> None:
    """One record's sparse posterior block.  `bpp` is the (L, L) upper-triangle
    matrix of `bpp` / `bpp_batch`; entry (i, j), i < j, is listed on line i + 1
    as `j+1:p` when p >= cutoff."""
    L = len(seq)
    mat = np.asarray(bpp, dtype=np.float64)
    if mat.shape != (L, L):
        raise ValueError(f"posterior matrix shape {mat.shape} != ({L}, {L})")
    if name is not None:
        fh.write(f">{name}\n")
    for i in range(L):
        row = mat[i, i + 1:]
        js = np.nonzero(row >= cutoff)[0]
        parts = [f"{i + 1}", seq[i]]
        parts.extend(f"{i + 2 + int(k)}:{row[k]:.6g}" for k in js)
        fh.write(" ".join(parts) + "\n")


def read_posteriors(path: str, n: int) -> np.ndarray:
    """(n, n) upper-triangle matrix from a single-record posteriors file, read
    the way the reference reads the binary's output (reference.py:112-125)."""
    mat = np.zeros((n, n), dtype=np.float64)
    with open(path) as fh:
        for line in fh:
            parts = line.split()
            if len(parts) < 2:
                continue
            i = int(parts[0]) - 1
            for tok in parts[2:]:
                j_s, p_s = tok.split(":")
                j = int(j_s) - 1
                if j > i:
                    mat[i, j] = float(p_s)
                else:
                    mat[j, i] = float(p_s)
    return mat


def write_parens_file(path: str, records: Iterable[Tuple[object, str, str]]) -> None:
    """Parens file of (name, seq, structure) records."""
    with open(path, "w") as fh:
        for name, seq, st in records:
            write_parens(fh, name, seq, st)


def write_posteriors_file(path: str, records: Iterable[Tuple[object, str, np.ndarray]], cutoff: float = 1e-5) -> None:
    """Posteriors file of (name, seq, bpp) records: a single record is written
    bare (the binary's layout); several get a `>name` line before each block."""
    recs = list(records)
    with open(path, "w") as fh:
        for name, seq, mat in recs:
            write_posteriors(fh, seq, mat, cutoff, name if len(recs) > 1 else None)
