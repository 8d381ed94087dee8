"""Radiometry converter (the format step before classify for real data):
an Erisyon radmat ([reads][channels][mocks + cycles], .npy or a flat .tsv)
to the whatprot radiometry TSV, as python/convert_radiometries.py does.

The output starts with the cycles, channels and reads counts, then one row
per read of cycles x channels values (cycle-major), the mock cycles left
out.  Values are written with Python's str(); like the reference, an entry
is preceded by a tab whenever its cycle or channel index is nonzero, so with
mock cycles every row starts with a tab (readers split on whitespace).
Optional ranges keep only reads whose every value lies strictly inside one
of its channel's (low, high) ranges.
"""
from __future__ import annotations

import sys
from typing import Optional, Sequence, Tuple

import numpy as np


def load_radmat(path: str, num_channels: int, num_mocks: int, num_cycles: int) -> Optional[np.ndarray]:
    ext = path.rsplit(".", 1)[-1]
    if ext == "npy":
        return np.load(path)
    if ext == "tsv":
        flat = np.genfromtxt(path, delimiter="\t", dtype=float)
        flat = np.atleast_2d(flat)
        return flat.reshape(flat.shape[0], num_channels, num_mocks + num_cycles)
    return None


def filter_ranges(radmat: np.ndarray, ranges_by_channel: Sequence[Sequence[Tuple[float, float]]]) -> np.ndarray:
    keep = np.ones(radmat.shape[0], dtype=bool)
    for c, ranges in enumerate(ranges_by_channel):
        x = radmat[:, c, :]
        ok = np.zeros_like(x, dtype=bool)
        for lo, hi in ranges:
            ok |= (lo < x) & (x < hi)
        keep &= ok.all(axis=1)
    return radmat[keep]


def convert_radiometries(num_channels: int, num_mocks: int, num_cycles: int, radmat_file: str, output_file: str,
                         ranges_by_channel=None) -> Optional[int]:
    """Returns the number of reads written (None for an unknown input type)."""
    radmat = load_radmat(radmat_file, num_channels, num_mocks, num_cycles)
    if radmat is None:
        return None
    print("Read " + str(radmat.shape[0]) + " radiometries.\n")
    if ranges_by_channel is not None:
        radmat = filter_ranges(radmat, ranges_by_channel)
        print("After filtering, " + str(radmat.shape[0]) + " radiometries remain.\n")
    rads = np.transpose(radmat, (0, 2, 1))  # [reads][cycles][channels]
    with open(output_file, "w") as f:
        f.write(f"{num_cycles}\n{num_channels}\n{rads.shape[0]}\n")
        for rad in rads:
            parts = []
            for i in range(num_mocks, num_mocks + num_cycles):
                for j in range(num_channels):
                    parts.append(("\t" if (i > 0 or j > 0) else "") + str(rad[i, j]))
            f.write("".join(parts) + "\n")
    return rads.shape[0]


if __name__ == "__main__":
    if len(sys.argv) != 6:
        print("usage: python -m whatprot_gb300.convert NUM_CHANNELS NUM_MOCKS NUM_CYCLES RADMAT OUTPUT")
        sys.exit(1)
    n = convert_radiometries(int(sys.argv[1]), int(sys.argv[2]), int(sys.argv[3]), sys.argv[4], sys.argv[5])
    sys.exit(0 if n is not None else 1)
