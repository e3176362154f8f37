"""A small GROMACS .xtc writer for tests: frames of integer (quantised)
coordinates encoded with the format's large-atom / small-run scheme, so the
decoders can be checked on paths the example trajectory may not reach
(natoms <= 9 raw frames, ranges above 2^24, runs, small-index changes, a
run length reused through a clear flag bit).

It writes the bit stream the decoders read: per group, the large atom as one
mixed-radix integer (or three fixed-width fields), a flag bit, optionally a
5-bit run field (3 * small atoms + is_smaller + 1), then the small atoms as
deltas of radix MAGIC[smallidx]; the first small atom of a run is placed
before the large atom in the decoded order.
"""
import struct

import numpy as np

MAGIC = [0, 0, 0, 0, 0, 0, 0, 0, 0, 8, 10, 12, 16, 20, 25, 32, 40, 50, 64, 80, 101, 128, 161, 203, 256, 322, 406,
         512, 645, 812, 1024, 1290, 1625, 2048, 2580, 3250, 4096, 5060, 6501, 8192, 10321, 13003, 16384, 20642, 26007,
         32768, 41285, 52015, 65536, 82570, 104031, 131072, 165140, 208063, 262144, 330280, 416127, 524287, 660561,
         832255, 1048576, 1321122, 1664510, 2097152, 2642245, 3329021, 4194304, 5284491, 6658042, 8388607, 10568983,
         13316085, 16777216]
FIRST = 9


class _Bits:
    def __init__(self):
        self.b = []

    def put(self, v, n):
        for i in range(n - 1, -1, -1):
            self.b.append((v >> i) & 1)

    def packed(self, v, n):  # little-endian 8-bit groups, the last one short
        while n > 8:
            self.put(v & 0xFF, 8)
            v >>= 8
            n -= 8
        if n > 0:
            self.put(v & ((1 << n) - 1), n)

    def tobytes(self):
        b = self.b + [0] * (-len(self.b) % 8)
        return bytes(int("".join(map(str, b[i:i + 8])), 2) for i in range(0, len(b), 8))


def _header(natoms, step, time, box):
    return struct.pack(">iiif", 1995, natoms, step, time) + struct.pack(">9f", *box) + struct.pack(">i", natoms)


def encode_frame(q, prec=1000.0, step=0, time=0.0, groups=None, smallidx=12, box=(3, 0, 0, 0, 3, 0, 0, 0, 3)):
    """q: int array [natoms, 3] (coordinate * prec). groups: list of
    (n_small, is_smaller, explicit_flag) per group, covering all atoms in
    order: a group emits n_small + 1 atoms; explicit_flag False reuses the
    previous group's run (its n_small must then equal the previous one's and
    is_smaller must be 0). Small deltas must fit the current radix.
    Returns the frame's bytes."""
    q = np.asarray(q, np.int64)
    n = len(q)
    if n <= 9:
        return _header(n, step, time, box) + struct.pack(">%df" % (3 * n), *(q.reshape(-1) / prec))
    if groups is None:
        groups = [(0, 0, True)] * n
    mn, mx = q.min(0), q.max(0)
    size = [int(v) for v in mx - mn + 1]
    large = any(s > 0xFFFFFF for s in size)
    bitsize = 0 if large else (size[0] * size[1] * size[2]).bit_length()
    w = _Bits()
    sidx = smallidx
    smaller = MAGIC[max(FIRST, sidx - 1)] // 2
    smallnum = MAGIC[sidx] // 2
    run = 0
    a = 0
    for ns, dsm, explicit in groups:
        seq = q[a:a + ns + 1]
        a += ns + 1
        big = seq[1] if ns > 0 else seq[0]
        v = [int(big[c] - mn[c]) for c in range(3)]
        if large:
            for c in range(3):
                w.put(v[c], size[c].bit_length())
        else:
            w.packed((v[0] * size[1] + v[1]) * size[2] + v[2], bitsize)
        if explicit:
            w.put(1, 1)
            w.put(3 * ns + dsm + 1, 5)
            run = 3 * ns
        else:
            assert run == 3 * ns and dsm == 0
            w.put(0, 1)
        m = MAGIC[sidx]
        order = ([seq[0]] + list(seq[2:])) if ns > 0 else []
        prev = big
        for t in order:
            d = [int(t[c] - prev[c] + smallnum) for c in range(3)]
            assert all(0 <= x < m for x in d), "small delta does not fit the radix"
            w.packed((d[0] * m + d[1]) * m + d[2], sidx)
            prev = t
        sidx += dsm
        if dsm < 0:
            smallnum = smaller
            smaller = MAGIC[sidx - 1] // 2 if sidx > FIRST else 0
        elif dsm > 0:
            smaller = smallnum
            smallnum = MAGIC[sidx] // 2
    assert a == n
    data = w.tobytes()
    out = _header(n, step, time, box) + struct.pack(">f", prec) + struct.pack(">3i", *mn) + struct.pack(">3i", *mx)
    out += struct.pack(">ii", smallidx, len(data)) + data + b"\0" * (-len(data) % 4)
    return out


def walk(natoms, seed, step=1):
    """Integer coordinates where consecutive atoms differ by at most `step`
    quanta per axis (so any small radix holds the deltas)."""
    rng = np.random.default_rng(seed)
    q = np.cumsum(rng.integers(-step, step + 1, size=(natoms, 3)), axis=0)
    return q + rng.integers(0, 5000, size=3)
