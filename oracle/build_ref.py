#!/usr/bin/env python3
"""Build recipe for ``oracle/_ref/ref_driver``: the reference's own C++ code for the
Monte Carlo path, compiled in this container to pin the CPU restatement and to
write the golden fixtures under ``tests/golden/``.

The reference ships as MSVC-flavoured C++17.  g++ 13 needs five mechanical,
semantics-preserving edits, applied to a transient copy under ``oracle/_ref/src``
that is deleted as soon as the binary is linked (no reference source is kept in
the tree or shipped anywhere):

1. ``mcBase.h`` / ``ThreadPool.cpp`` include ``ThreadPool.h``; the file is ``threadPool.h``.
2. ``AADExpr.h`` calls member templates of dependent objects without the
   ``template`` keyword (``x.pushAdjoint<N, n>(...)``).
3. ``mcBase.h`` explicitly specialises a member template inside the class
   (``putParametersOnTapeT<Number>``); rewritten as ``if constexpr``.
4. ``mrg32k3a.h`` uses functional casts spelled ``unsigned long long(x)``.
5. ``std::memset`` / ``std::mem_fn`` are used without their headers
   (solved with ``-include cstring -include functional``).

Translation units: ``AAD.cpp mcBase.cpp ThreadPool.cpp sobol.cpp`` plus the
driver ``oracle/ref_driver.cpp`` (which includes ``main.h`` once).  Flags:
``-std=c++17 -O2 -ffp-contract=off``; no ``-ffast-math`` (the reference's own
project uses ``/fp:fast``; the oracle must not).

Usage: ``python3 oracle/build_ref.py --reference DIR`` (or ``CF_REFERENCE_DIR=DIR``).  Exit status 0 and the
binary path on stdout on success; exit status 2 when the reference is absent.
"""
import argparse
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")

# Files of the reference the path needs (headers + the four translation units).
FILES = [
    "AAD.h", "AADExpr.h", "AADNode.h", "AADNumber.h", "AADTape.h", "blocklist.h",
    "ConcurrentQueue.h", "analytics.h", "choldc.h", "gaussians.h", "interp.h", "ivs.h",
    "main.h", "matrix.h", "mcBase.h", "mcMdl.h", "mcMdlBS.h", "mcMdlDupire.h",
    "mcMdlMultiDisplaced.h", "mcPrd.h", "mcPrdMulti.h", "mrg32k3a.h", "sobol.h",
    "store.h", "threadPool.h", "utility.h",
    "AAD.cpp", "mcBase.cpp", "ThreadPool.cpp", "sobol.cpp",
]
TUS = ["AAD.cpp", "mcBase.cpp", "ThreadPool.cpp", "sobol.cpp"]


def _patch(src_dir):
    def edit(name, fn):
        p = os.path.join(src_dir, name)
        with open(p, encoding="latin-1") as f:
            s = f.read()
        t = fn(s)
        if t == s:
            raise SystemExit(f"build_ref: patch for {name} did not apply")
        with open(p, "w", encoding="latin-1") as f:
            f.write(t)

    # (1) include case
    edit("mcBase.h", lambda s: s.replace('#include "ThreadPool.h"', '#include "threadPool.h"'))
    edit("ThreadPool.cpp", lambda s: s.replace('#include "ThreadPool.h"', '#include "threadPool.h"'))
    # (2) missing `template` keyword on dependent member-template calls
    edit("AADExpr.h", lambda s: re.sub(r"\.pushAdjoint<", ".template pushAdjoint<", s))
    # (3) in-class explicit specialisation -> if constexpr in the primary template
    def fix_spec(s):
        pat = re.compile(
            r"template<class U>\s*\n\s*void putParametersOnTapeT\(\)\s*\{\s*\}\s*"
            r"(//[^\n]*\n\s*)?template <>\s*\n\s*void putParametersOnTapeT<Number>\(\)\s*\{(.*?)\}\s*\n",
            re.S)
        repl = ("template<class U>\n    void putParametersOnTapeT()\n    {\n"
                "        if constexpr (std::is_same_v<U, Number>)\n        {\\2}\n    }\n")
        return pat.sub(repl, s, count=1)
    edit("mcBase.h", fix_spec)
    # (4) functional casts with a multi-word type name
    edit("mrg32k3a.h", lambda s: re.sub(r"unsigned long long\s*\(", "(unsigned long long)(", s))


def build(reference):
    if not os.path.isdir(reference):
        print(f"build_ref: reference not found at {reference}", file=sys.stderr)
        return 2
    src = os.path.join(OUT, "src")
    if os.path.isdir(src):
        shutil.rmtree(src)
    os.makedirs(src)
    try:
        for f in FILES:
            shutil.copy(os.path.join(reference, f), os.path.join(src, f))
        _patch(src)
        objs = []
        cmds = []
        for tu in TUS + [os.path.join(HERE, "ref_driver.cpp")]:
            base = os.path.splitext(os.path.basename(tu))[0]
            obj = os.path.join(OUT, base + ".o")
            path = tu if os.path.isabs(tu) else os.path.join(src, tu)
            cmds.append(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-w",
                         "-include", "cstring", "-include", "functional",
                         "-I", src, "-c", path, "-o", obj])
            objs.append(obj)
        procs = [subprocess.Popen(c) for c in cmds]
        rcs = [p.wait() for p in procs]
        if any(rcs):
            print("build_ref: compile failed", file=sys.stderr)
            return 1
        exe = os.path.join(OUT, "ref_driver")
        rc = subprocess.call(["g++", "-O2", "-o", exe] + objs + ["-lpthread"])
        for o in objs:
            os.remove(o)
        if rc:
            return 1
        print(exe)
        return 0
    finally:
        shutil.rmtree(src, ignore_errors=True)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("CF_REFERENCE_DIR"),
                    help="the reference checkout (or CF_REFERENCE_DIR); required")
    a = ap.parse_args()
    if not a.reference:
        ap.error("the reference checkout is required: --reference DIR or CF_REFERENCE_DIR")
    sys.exit(build(a.reference))
