#!/usr/bin/env python3
"""Derive the Joe-Kuo initialisation data (degree s, polynomial bits a, initial m_1..m_s)
of each Sobol dimension from the expanded direction-number table of the reference
(sobol.cpp: 32 direction numbers x 1111 dimensions, Joe & Kuo's "old" 1111-dimension set).

The library regenerates the full table from this compact data with the Joe-Kuo
recurrence (compfinance_gb300/csrc/host_math.cpp), so the points are bit-identical
without carrying the expanded table.  An offline recipe: it reads the reference's
sobol.cpp, whose path is a required argument.  Usage:

    python3 oracle/derive_sobol_init.py REFERENCE_DIR/sobol.cpp > compfinance_gb300/data/sobol_joe_kuo.inc

The output is a C/C++ initializer list included by the library and by the oracle.
"""
import re
import sys


def parse(path):
    txt = open(path, encoding="latin-1").read()
    dirs = []
    for i in range(1, 33):
        m = re.search(r"const unsigned jkDir%d\[\]\s*=\s*\{(.*?)\};" % i, txt, re.S)
        dirs.append([int(x) for x in m.group(1).replace("\n", " ").split(",") if x.strip()])
    return dirs  # dirs[i][d]


def regen(s, a, m):
    """Joe-Kuo recurrence: m_k = 2a_1 m_{k-1} ^ 4a_2 m_{k-2} ^ ... ^ 2^s m_{k-s} ^ m_{k-s}."""
    m = list(m)
    for k in range(s, 32):
        v = m[k - s] ^ (m[k - s] << s)
        for j in range(1, s):
            if (a >> (s - 1 - j)) & 1:
                v ^= m[k - j] << j
        m.append(v)
    return [m[k] << (31 - k) for k in range(32)]


def derive(col):
    mk = [col[k] >> (31 - k) for k in range(32)]
    for s in range(1, 20):
        for a in range(1 << (s - 1)):
            if regen(s, a, mk[:s]) == col:
                return s, a, mk[:s]
    raise SystemExit("no recurrence found")


def main():
    if len(sys.argv) != 2:
        raise SystemExit("usage: python3 oracle/derive_sobol_init.py REFERENCE_DIR/sobol.cpp")
    path = sys.argv[1]
    dirs = parse(path)
    ndim = len(dirs[0])
    print("/* Joe-Kuo Sobol initialisation data ('old' set), %d dimensions." % ndim)
    print(" * One entry per dimension: {s, a, {m_1, ..., m_s}}; dimension 0 is van der Corput (s=0).")
    print(" * Generated by oracle/derive_sobol_init.py. */")
    print("#define CF_SOBOL_MAX_DIM %d" % ndim)
    for d in range(ndim):
        col = [dirs[i][d] for i in range(32)]
        if all(col[k] == 1 << (31 - k) for k in range(32)):
            print("{0, 0, {0}},")
            continue
        s, a, m = derive(col)
        print("{%d, %d, {%s}}," % (s, a, ", ".join(str(x) for x in m)))


if __name__ == "__main__":
    main()
