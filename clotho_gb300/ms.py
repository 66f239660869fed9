"""Hudson's `ms` output format for samples of a population.

The reference's analysis tools read samples in this format
(src/tools/ms/ms_allele_freq.py: a header up to the first blank line, then per
replicate `//`, `segsites: S`, `positions: ...` and one 0/1 string of length S
per sequence).  `write_ms` writes the segregating sites of a sample of rows,
columns ordered by allele position (ties by slot); `read_ms` parses such text.
"""
from __future__ import annotations

import io

import numpy as np


def sample_matrix(rows: np.ndarray, A: int, sample=None):
    """0/1 matrix [n x A] of the sampled rows (reference bit layout: slot a is
    bit a%64 of word a/64)."""
    rows = np.asarray(rows, np.uint64)
    if sample is not None:
        rows = rows[np.asarray(sample, np.int64)]
    bits = np.unpackbits(rows.view(np.uint8).reshape(rows.shape[0], -1), axis=1, bitorder="little")
    return bits[:, :A]


def segregating_columns(hap: np.ndarray, positions: np.ndarray):
    """Slots segregating in the sample, ordered by position then slot."""
    n = hap.shape[0]
    cnt = hap.sum(axis=0) if hap.size else np.zeros(hap.shape[1], np.int64)
    seg = np.nonzero((cnt > 0) & (cnt < n))[0]
    order = np.lexsort((seg, np.asarray(positions)[seg]))
    return seg[order]


def write_ms(fp, rows: np.ndarray, positions, sample=None, command: str = "clotho_gb300",
             seeds=(0, 0, 0), precision: int = 10, header: bool = True):
    """Write one replicate of the sampled rows.  Returns the slots written, in column order."""
    positions = np.asarray(positions, np.float64)
    hap = sample_matrix(rows, positions.size, sample)
    cols = segregating_columns(hap, positions)
    out = io.StringIO()
    if header:
        out.write(f"{command}\n{' '.join(str(int(s)) for s in seeds)}\n\n")
    out.write("//\n")
    out.write(f"segsites: {cols.size}\n")
    if cols.size:
        out.write("positions: " + " ".join(f"{positions[c]:.{precision}f}" for c in cols) + "\n")
        sub = hap[:, cols].astype(np.uint8) + ord("0")
        for r in sub:
            out.write(r.tobytes().decode() + "\n")
    out.write("\n")
    fp.write(out.getvalue())
    return cols


def read_ms(text: str):
    """Replicates of an ms file: [{"segsites", "positions", "haplotypes" (n x S uint8)}]."""
    lines = text.split("\n")
    i = 0
    while i < len(lines) and lines[i].strip():  # header up to the first blank line
        i += 1
    reps = []
    while i < len(lines):
        if not lines[i].startswith("//"):
            i += 1
            continue
        i += 1
        S = int(lines[i].split(":")[1])
        i += 1
        pos = np.zeros(0)
        if S:
            pos = np.array([float(x) for x in lines[i].split(":")[1].split()])
            i += 1
        haps = []
        while i < len(lines) and lines[i].strip() and not lines[i].startswith("//"):
            if S:
                haps.append(np.frombuffer(lines[i].strip().encode(), np.uint8) - ord("0"))
            i += 1
        hap = np.array(haps, np.uint8).reshape(len(haps), S) if haps else np.zeros((0, S), np.uint8)
        reps.append({"segsites": S, "positions": pos, "haplotypes": hap})
    return reps
