"""CPU restatement of GAMMCOR's AO integral sort (readtwoint).

TEST INFRASTRUCTURE ONLY (the oracle of gc_sort_twoint): only tests/ import it.
Integer and byte work: the GPU result must match it bit for bit.

readtwoint (sorter.f90:31-395) decodes each integral's labels, adds it to the
bucket of record rs at element pq (add_to_Sorter, sorter.f90:456-472) and, by
the format's rule, to the bucket of record pq at element rs; SORT2
(get_from_Sorter, sorter.f90:517-539) starts every record at zero and replays
its bucket in order, so a slot written twice keeps the later integral.
"""
from __future__ import annotations

import numpy as np


def _tri1(p, q):  # 1-based packed pair index, p <= q
    return p + q * (q - 1) // 2


def placements(fmt: str, labels, t: int):
    """[(rs, pq), ...] of integral t, 1-based, in the reference's add order."""
    if fmt == "dalton8":                                  # sorter.f90:84-104
        x = int(labels[t]) & 0xFFFFFFFF
        p, q, r, s = x & 255, (x >> 8) & 255, (x >> 16) & 255, (x >> 24) & 255
        pq, rs = p + q * (q - 1) // 2, r + s * (s - 1) // 2
        return [(rs, pq)] + ([(pq, rs)] if pq < rs else [])
    if fmt == "dalton16":                                 # sorter.f90:106-125
        a, b = int(labels[2 * t]) & 0xFFFFFFFF, int(labels[2 * t + 1]) & 0xFFFFFFFF
        r, s, p, q = a & 65535, a >> 16, b & 65535, b >> 16
        pq, rs = p + q * (q - 1) // 2, r + s * (s - 1) // 2
        return [(rs, pq)] + ([(pq, rs)] if pq < rs else [])
    if fmt == "pqrs":                                     # sorter.f90:303-318
        p, q, r, s = (int(v) for v in labels[4 * t:4 * t + 4])
        pq = _tri1(min(p, q), max(p, q))
        rs = _tri1(min(r, s), max(r, s))
        return [(rs, pq), (pq, rs)]
    raise ValueError(fmt)


def readtwoint(nbas: int, values, labels, fmt: str, out=None):
    """AOTWOSORT tensor (ntr, ntr), out[rs-1, pq-1] = (pq|rs)."""
    ntr = nbas * (nbas + 1) // 2
    if out is None:
        out = np.zeros((ntr, ntr))
    if fmt == "triangle":                                 # sorter.f90:324-345
        t = 0
        pq = 0
        for p in range(1, nbas + 1):
            for q in range(1, p + 1):
                pq += 1
                rs = 0
                for r in range(1, nbas + 1):
                    for s in range(1, r + 1):
                        rs += 1
                        if pq >= rs:
                            out[rs - 1, pq - 1] = values[t]
                            out[pq - 1, rs - 1] = values[t]
                            t += 1
        return out
    for t in range(len(values)):
        for rs, pq in placements(fmt, labels, t):
            if 1 <= rs <= ntr and 1 <= pq <= ntr:
                out[rs - 1, pq - 1] = values[t]
    return out
