"""Compiles reference OKL kernels for the CPU with OCCA's Serial-mode semantics
(test infrastructure: the output pins the oracle; the library never uses it).

The reference's gather-scatter, Jacobi, vector, dot and adv kernels exist only
as OKL (``.okl``), which the OCCA runtime translates at run time.  This recipe
reads the unmodified ``.okl`` files from the nekBench source tree, applies the
Serial backend's meaning of each OKL attribute and compiles the result with
g++ into ``oracle/_ref/`` (git-ignored):

* ``@kernel``              -> an ``extern "C"`` function (arguments as written)
* ``for(...; @outer(n))``  -> a plain loop
* ``for(...; @inner(n))``  -> a plain loop; nested inner loops run in order,
                              one "thread" after another
* ``for(...; @tile(T, @outer, @inner))`` -> a plain loop over the same range
* ``@shared``              -> an ordinary local array of the outer iteration
* ``@exclusive``           -> one copy per inner iteration: an array indexed by
                              a counter that restarts at every inner-loop nest
                              and advances after each innermost iteration
* ``@barrier(...)``        -> nothing (inner loops already run to completion)
* ``@restrict``            -> nothing (an aliasing hint written before the type,
                              where C++ does not accept one)

Compile-time constants are the ``-D`` defines the reference's drivers pass
(``p_Nq``, ``p_blockSize`` ...) plus ``core/params.h``; ``-ffp-contract=off``
keeps the arithmetic exactly as written.

  python oracle/okl_serial.py --tree <nekBench source tree>   (or NEKB_REFERENCE)
"""
from __future__ import annotations

import argparse
import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
EXMAX = 1024  # inner iterations per outer iteration an exclusive variable covers


def strip_comments(src: str) -> str:
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    return re.sub(r"//[^\n]*", "", src)


def match_close(s: str, i: int, open_ch: str, close_ch: str) -> int:
    """Index just past the bracket that closes s[i] (== open_ch)."""
    depth = 0
    for k in range(i, len(s)):
        if s[k] == open_ch:
            depth += 1
        elif s[k] == close_ch:
            depth -= 1
            if depth == 0:
                return k + 1
    raise ValueError("unbalanced " + open_ch)


def split_top(s: str, sep: str) -> list:
    parts, depth, cur = [], 0, []
    for ch in s:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == sep and depth == 0:
            parts.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    parts.append("".join(cur))
    return parts


def skip_ws(s: str, i: int) -> int:
    while i < len(s) and s[i].isspace():
        i += 1
    return i


def statement_end(s: str, i: int) -> int:
    """Index just past the statement starting at s[i] (block, for/if/while or
    an expression statement); loop markers written by this recipe are skipped."""
    i = skip_ws(s, i)
    while s.startswith("/*", i):
        i = skip_ws(s, s.index("*/", i) + 2)
    if s[i] == "{":
        return match_close(s, i, "{", "}")
    if s.startswith("#", i):  # a preprocessor line
        return s.index("\n", i) + 1
    m = re.match(r"(for|while)\s*\(", s[i:])
    if m:
        h = match_close(s, i + m.end() - 1, "(", ")")
        return statement_end(s, h)
    m = re.match(r"if\s*\(", s[i:])
    if m:
        h = match_close(s, i + m.end() - 1, "(", ")")
        e = statement_end(s, h)
        j = skip_ws(s, e)
        if re.match(r"else\b", s[j:]):
            return statement_end(s, j + 4)
        return e
    depth = 0
    for k in range(i, len(s)):
        if s[k] in "([{":
            depth += 1
        elif s[k] in ")]}":
            depth -= 1
        elif s[k] == ";" and depth == 0:
            return k + 1
    raise ValueError("statement without end")


def extract_kernel(src: str, name: str) -> str:
    m = re.search(r"@kernel\s+void\s+" + re.escape(name) + r"\s*\(", src)
    if not m:
        raise KeyError(name)
    args_end = match_close(src, m.end() - 1, "(", ")")
    body = src.index("{", args_end)
    return src[m.start():match_close(src, body, "{", "}")]


def translate(kernel: str) -> str:
    k = kernel.replace("@kernel", 'extern "C"').replace("@restrict", "")
    k = re.sub(r"@barrier\s*\([^)]*\)\s*;", ";", k)
    k = re.sub(r"@shared\b", "", k)
    # @exclusive declarations -> arrays with one slot per inner iteration
    excl = []

    def excl_decl(m):
        decl = m.group(1).strip()
        tm = re.match(r"((?:const\s+)?\w+)\s+(.*)", decl, flags=re.S)
        typ, rest = tm.group(1), tm.group(2)
        outs = []
        for d in split_top(rest, ","):
            dm = re.match(r"\s*(\w+)\s*(.*)", d, flags=re.S)
            excl.append(dm.group(1))
            outs.append(f"{dm.group(1)}@EX@{dm.group(2).strip()}")
        return f"{typ} " + ", ".join(outs) + ";"

    k = re.sub(r"@exclusive\s+([^;]+);", excl_decl, k)
    for nm in excl:
        k = re.sub(r"\b" + nm + r"\b(?!@EX@)", nm + "[__ex]", k)
    k = k.replace("@EX@", f"[{EXMAX}]")
    # annotated loops: rewrite headers, mark inner loops
    out, i = [], 0
    pat = re.compile(r"\bfor\s*\(")
    while True:
        m = pat.search(k, i)
        if not m:
            out.append(k[i:])
            break
        h0, h1 = m.end() - 1, match_close(k, m.end() - 1, "(", ")")
        parts = split_top(k[h0 + 1:h1 - 1], ";")
        if len(parts) == 4:
            attr = parts[3].strip()
            out.append(k[i:m.start()])
            kind = "inner0" if re.match(r"@inner\s*\(\s*0\s*\)", attr) else \
                   "inner" if attr.startswith("@inner") else "plain"
            out.append(f"for({parts[0]};{parts[1]};{parts[2]}) /*{kind}*/")
            i = h1
        else:
            out.append(k[i:h1])
            i = h1
    k = "".join(out)
    if excl:
        # wrap innermost inner bodies with the counter step; reset the counter
        # before every inner-loop nest
        k = wrap_inner(k)
        body = k.index("{")
        k = k[:body + 1] + "\n  int __ex = 0; (void)__ex;\n" + k[body + 1:]
    return k


def loop_spans(k: str) -> list:
    """(start, end, kind, header_end) of every marked loop."""
    spans = []
    for m in re.finditer(r"\bfor\s*\(", k):
        h1 = match_close(k, m.end() - 1, "(", ")")
        mm = re.match(r"\s*/\*(inner0|inner|plain)\*/", k[h1:])
        if mm:
            spans.append((m.start(), statement_end(k, h1), mm.group(1), h1 + mm.end()))
    return spans


def wrap_inner(k: str) -> str:
    # innermost loops (@inner(0)): body -> { body ++__ex; }
    for s0, e, kind, b0 in sorted(loop_spans(k), reverse=True):
        if kind == "inner0":
            k = k[:b0] + " { " + k[b0:e] + "\n ++__ex; }" + k[e:]
    # the counter restarts before the outermost loop of every inner nest
    inner = [(s0, e) for s0, e, kind, _ in loop_spans(k) if kind in ("inner", "inner0")]
    starts = [s0 for s0, e in inner if not any(s2 < s0 < e2 for s2, e2 in inner)]
    for s0 in sorted(starts, reverse=True):
        k = k[:s0] + "__ex = 0; " + k[s0:]
    return k


def build(tree: str, okl: str, kernels: list, defines: dict, tag: str, verbose=False) -> str:
    """Translate `kernels` of tree/okl with `defines`; returns the .so path."""
    src = strip_comments(open(os.path.join(tree, okl)).read())
    # keep the file's own #define lines (they precede or sit inside kernels)
    code = [translate(extract_kernel(src, k)) for k in kernels]
    os.makedirs(OUT, exist_ok=True)
    cpp = os.path.join(OUT, f"okl_{tag}.cpp")
    with open(cpp, "w") as f:
        f.write(f"// generated by oracle/okl_serial.py from {okl}; do not edit\n")
        f.write("#include <math.h>\n")
        f.write("\n\n".join(code) + "\n")
    so = os.path.join(OUT, f"libokl_{tag}.so")
    cmd = ["g++", "-O2", "-fPIC", "-shared", "-w", "-ffp-contract=off", "-x", "c++",
           "-include", os.path.join(tree, "core", "params.h")]
    cmd += [f"-D{k}={v}" for k, v in defines.items()]
    cmd += [cpp, "-o", so]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return so


# the kernels this repository pins, with the defines their drivers pass
def targets(Nq_list=(4, 8), block_sizes=(256, 512, 1024)):
    base = {"dfloat": "double", "dlong": "int"}
    t = []
    t.append(("gs", "3rdParty/ogs/okl/gatherScatterMany.okl", ["gatherScatterMany_doubleAdd"], base))
    for nq in Nq_list:
        t.append((f"jacobi_nq{nq}", "nekBone/kernel/updateJacobi.okl", ["updateJacobi"],
                  {**base, "p_Nq": nq, "p_Np": nq ** 3}))
    for nf in (1, 3):
        t.append((f"utils_nf{nf}", "nekBone/kernel/utils.okl",
                  ["weightedInnerProductUpdate", "BPUpdatePCG"],
                  {**base, "p_blockSize": 256, "p_Nfields": nf}))
    for bs in block_sizes:
        t.append((f"dot_bs{bs}", "dot/kernel/VOLTA/dot.okl",
                  ["weightedInnerProduct2_v0", "weightedBlockInnerProduct2",
                   "weightedInnerProduct2_v1"],
                  {**base, "p_blockSize": bs, "p_eNfields": 1}))
    for nq in Nq_list:
        adv = {**base, "p_Nq": nq, "p_cubNq": nq, "p_Np": nq ** 3, "p_cubNp": nq ** 3,
               "p_Nvgeo": 12, "p_RXID": 0, "p_RYID": 1, "p_SXID": 2, "p_SYID": 3, "p_JID": 4,
               "p_JWID": 5, "p_IJWID": 6, "p_RZID": 7, "p_SZID": 8, "p_TXID": 9, "p_TYID": 10,
               "p_TZID": 11}
        t.append((f"adv_nq{nq}", "adv/kernel/VOLTA/adv.okl", ["advCubatureHex3D_v0"], adv))
    return t


def main():
    ap = argparse.ArgumentParser(description="OKL kernels of the reference, Serial semantics")
    ap.add_argument("--tree", default=os.environ.get("NEKB_REFERENCE", ""))
    ap.add_argument("-v", action="store_true")
    a = ap.parse_args()
    if not a.tree or not os.path.isdir(a.tree):
        raise SystemExit("okl_serial: give --tree or set NEKB_REFERENCE to the nekBench source tree")
    for tag, okl, kernels, defines in targets():
        print(build(a.tree, okl, kernels, defines, tag, a.v))


if __name__ == "__main__":
    main()
