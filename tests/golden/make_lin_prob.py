"""Convert the reference's solver fixture into tests/golden/lin_prob.npz.

Reads algo/linear_solver/test/lin_prob.xml.bz2 from the reference tree (an
iotk binary file: Fortran sequential records, each data record carrying a
4-byte prefix before its payload) and stores DIMENSION, LIST_SHIFT,
LINEAR_OPERATOR (column-major n x n) and RIGHT_HAND_SIDE.  The solver test
(linear_solver.pf:125-345) reads the same four items.  Run once, with the
path of a reference checkout:
    python tests/golden/make_lin_prob.py <reference checkout>
"""
import bz2
import os
import re
import struct
import sys

import numpy as np


def read_iotk(path):
    raw = bz2.open(path, "rb").read()
    recs, p = [], 0
    while p < len(raw):
        (ln,) = struct.unpack_from("<i", raw, p)
        recs.append(raw[p + 4:p + 4 + ln])
        p += 8 + ln
    out, i = {}, 0
    while i < len(recs):
        m = re.search(rb'<(\w+) type="(\w+)" size="(\d+)" kind="(\d+)"', recs[i])
        if m:
            name, typ, size, kind = m.group(1).decode(), m.group(2).decode(), int(m.group(3)), int(m.group(4))
            payload = recs[i + 1][4:]
            dt = {"integer": "<i%d" % kind, "complex": "<c%d" % (2 * kind), "real": "<f%d" % kind}[typ]
            out[name] = np.frombuffer(payload, dtype=dt, count=size).copy()
            i += 2
            continue
        i += 1
    return out


def main(ref_root):
    d = read_iotk(os.path.join(ref_root, "algo/linear_solver/test/lin_prob.xml.bz2"))
    n = int(d["DIMENSION"][0])
    a = d["LINEAR_OPERATOR"].reshape(n, n, order="F")
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lin_prob.npz")
    np.savez_compressed(out, A=a, b=d["RIGHT_HAND_SIDE"], sigma=d["LIST_SHIFT"])
    print("wrote", out, "n =", n, "shifts =", d["LIST_SHIFT"].size)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_lin_prob.py <reference checkout>")
    main(sys.argv[1])
