"""Writes tests/golden/reference_ccalls.json: the signatures with which the reference's
Julia code ccalls the native symbols of the path this library replaces, and the C++
signatures of the op functions behind its TensorFlow custom ops (deps/MFEM/*/*.h).

AdFem.jl calls its C++ library through `@eval ccall((:sym, $LIBMFEM), Ret, (ArgTypes...),
args...)` (src/MFEM/MFEM.jl, src/MFEM/MCore.jl, src/MFEM/MUtils.jl, src/pcl.jl).  This
script reads those call sites from a checkout of the reference and keeps every call whose
symbol include/adfem_gpu.h declares, with the file:line of the call.  Only the interface is
recorded (symbol, return type, argument types), so the drop-in test
(tests/test_binding_signatures_cpu.py) checks the header against the reference's own callers
without reading the reference at test time.

Run from the repository root:  python tests/golden/make_reference_ccalls.py [REFERENCE_DIR]
(default REFERENCE_DIR: /root/reference).
"""
import glob
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from test_binding_signatures_cpu import header_functions, julia_ccalls  # noqa: E402


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    declared = header_functions()
    calls = []
    for path in sorted(glob.glob(os.path.join(ref, "src", "**", "*.jl"), recursive=True)):
        text = open(path).read()
        rel = os.path.relpath(path, ref)
        for sym, ret, args in julia_ccalls(text):
            if sym not in declared:
                continue
            # line of the call site: first line that names the symbol in a ccall
            line = next(k + 1 for k, ln in enumerate(text.splitlines()) if "ccall((:%s," % sym in ln)
            calls.append({"symbol": sym, "returns": ret, "args": args, "site": "%s:%d" % (rel, line)})
    # the op functions (forward / backward / Julia entry / PCL helper) defined in the
    # reference's headers of the path, for the names this library exports: parameter types
    # in order, int64 written as the reference writes it
    ops = []
    for path in sorted(glob.glob(os.path.join(ref, "deps", "MFEM", "*", "*.h"))):
        text = open(path).read()
        rel = os.path.relpath(path, ref)
        for m in re.finditer(r"(?:extern \"C\"\s+)?void\s+(?:\w+::)?(\w+)\s*\(([^)]*)\)\s*\{", text):
            name = m.group(1)
            if name not in declared:
                continue
            params = [" ".join(p.split()) for p in m.group(2).split(",") if p.strip()]
            types = [re.sub(r"\s*\b\w+$", "", p).replace(" *", "*").replace("* ", "*").strip() for p in params]
            line = text[:m.start()].count("\n") + 1
            ops.append({"symbol": name, "params": types, "site": "%s:%d" % (rel, line)})
    out = os.path.join(HERE, "reference_ccalls.json")
    with open(out, "w") as fh:
        json.dump({"what": "ccall signatures of the reference's Julia callers for the symbols this library "
                           "exports (symbol, Julia return type, Julia argument types, call site), and the "
                           "C++ parameter types of the reference's op functions of the same names",
                   "calls": calls, "ops": ops}, fh, indent=1)
        fh.write("\n")
    print("wrote %s: %d call sites, %d op functions" % (out, len(calls), len(ops)))


if __name__ == "__main__":
    main()
