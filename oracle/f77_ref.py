"""Builds the reference's own (T) code for the CPU, by mechanical translation.

TEST INFRASTRUCTURE ONLY (checker side).  No Fortran compiler exists on this
machine or on the GPU host, so the reference's Fortran cannot be compiled
as it is.  src/tce/ccsd_t/ccsd_t_kernels_omp.F (the 27 sd_t_* kernels) and
src/tce/ccsd_t/ccsd_t_dot.F (the energy sum) are written in a small Fortran
subset -- declarations, DO loops, IF blocks, assignments -- and this script
translates that subset statement by statement into C (column-major array
addressing, by-reference arguments), then compiles it with gcc.  The
driver-side files src/tce/ccsd_t/ccsd_t_neword.F (the tuple list and its
weight order), src/tce/sort/tce_sort4.F and src/tce/sort/tce_sort2.F (the
block permutations) add integer arrays, an integer function, PARAMETERs,
labels with GOTO, CALLs and an early RETURN; they are translated in a
second mode with every scalar argument by reference (the reference's own
argument semantics), the Global Arrays rank queries ga_nodeid/ga_nnodes
answering 0 and 1 (one process), errquit aborting, and WRITE / FORMAT and
the cpusecs timers dropped.  The arithmetic and loop order are the
reference's own; nothing is restated by hand.  The sources are read where
they lie (the NWChem tree) and the output goes to oracle/_ref/, which is
not committed.

    python oracle/f77_ref.py [NWCHEM_SOURCE_TREE]

The tree is the argument, else the NWCHEM_SRC environment variable, else
the location this build's container mounts it at.

Preprocessing: the files are run through the C preprocessor in traditional
mode with no macros defined, which takes the reference's generic branches
(not CRAYFTN, not __ppc64__, no OpenMP directives; OpenMP directives are
comment lines in any case).
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
DEFAULT_TREE = Path(os.environ.get("NWCHEM_SRC", "/root/reference"))
FILES = ["src/tce/ccsd_t/ccsd_t_kernels_omp.F", "src/tce/ccsd_t/ccsd_t_dot.F"]
DRIVER_FILES = ["src/tce/ccsd_t/ccsd_t_neword.F", "src/tce/sort/tce_sort4.F", "src/tce/sort/tce_sort2.F"]
# Include files of the driver sources; they declare Global Arrays / MA
# interfaces and timers this translation does not use, so empty ones stand in.
STUB_INCLUDES = ["errquit.fh", "mafdecls.fh", "global.fh", "util.fh", "tce_main.fh"]


def preprocess(path: Path) -> list[str]:
    OUT.mkdir(exist_ok=True)
    inc = OUT / "stub_include"
    inc.mkdir(exist_ok=True)
    for name in STUB_INCLUDES:
        (inc / name).write_text("")
    res = subprocess.run(["cpp", "-P", "-traditional-cpp", "-I", str(inc), str(path)], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(res.stderr)
    return res.stdout.splitlines()


def statements(lines: list[str]) -> list[str]:
    """Fixed-form Fortran: drop comments, join continuation lines."""
    out: list[str] = []
    for ln in lines:
        if not ln.strip():
            continue
        if ln[0] in "cC*!" or ln.lstrip().startswith("!"):
            continue
        if len(ln) > 5 and ln[5] not in " 0" and ln[:5].strip() == "":
            out[-1] += " " + ln[6:].strip()
            continue
        code = ln[6:] if len(ln) > 6 else ""
        code = code.split("!")[0].rstrip()
        label = ln[:5].strip()
        if code.strip():
            out.append((f"@{label} " if label.isdigit() else "") + code.strip())
    return out


class Unit:
    def __init__(self, name: str, args: list[str], function: bool = False):
        self.name, self.args, self.function = name, args, function
        self.ints: set[str] = set()
        self.logicals: set[str] = set()
        self.doubles: dict[str, list[str]] = {}  # name -> dims (empty: scalar)
        self.intarrs: dict[str, list[str]] = {}  # integer arrays: name -> dims
        self.params: dict[str, str] = {}         # PARAMETER constants
        self.body: list[str] = []


DECL = re.compile(r"^(integer|double precision|logical)\s+(.*)$", re.I)


def split_top(s: str) -> list[str]:
    """Split a comma list at depth 0."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def parse(stmts: list[str], driver: bool = False) -> list[Unit]:
    units: list[Unit] = []
    u = None
    for st in stmts:
        low = st.lower()
        m = re.match(r"^(integer\s+function|subroutine)\s+(\w+)\s*\((.*)\)\s*$", st, re.I)
        if m:
            u = Unit(m.group(2).lower(), [a.strip().lower() for a in m.group(3).split(",")],
                     function=m.group(1).lower().startswith("integer"))
            units.append(u)
            continue
        if u is None:
            continue
        if low == "implicit none" or (low == "return" and not driver):
            continue
        if low == "end":
            u = None
            continue
        m = re.match(r"^parameter\s*\((\w+)\s*=\s*(.+)\)$", st, re.I)
        if m:
            u.params[m.group(1).lower()] = m.group(2).strip()
            continue
        m = DECL.match(st)
        if m:
            kind = m.group(1).lower()
            for item in split_top(m.group(2)):
                mm = re.match(r"^(\w+)\s*(?:\((.*)\))?$", item)
                name = mm.group(1).lower()
                dims = [d.strip().lower() for d in split_top(mm.group(2))] if mm.group(2) else []
                if kind == "integer" and dims:
                    u.intarrs[name] = dims
                elif kind == "integer":
                    u.ints.add(name)
                elif kind == "logical":
                    u.logicals.add(name)
                else:
                    u.doubles[name] = dims
            continue
        u.body.append(st)
    return units


def expr(e: str, u: Unit) -> str:
    """Fortran expression -> C: array references, logical operators, literals."""
    e = re.sub(r"(\d+\.\d*)d([+-]?\d+)", r"\1e\2", e, flags=re.I)
    e = re.sub(r"(\d+)d([+-]?\d+)", r"\1.0e\2", e, flags=re.I)
    for a, b in ((".eq.", "=="), (".ne.", "!="), (".and.", "&&"), (".or.", "||"), (".not.", "!"),
                 (".lt.", "<"), (".le.", "<="), (".gt.", ">"), (".ge.", ">=")):
        e = re.sub(re.escape(a), f" {b} ", e, flags=re.I)
    out, i = "", 0
    while i < len(e):
        m = re.match(r"[A-Za-z_]\w*", e[i:])
        if not m:
            out += e[i]
            i += 1
            continue
        name = m.group(0).lower()
        j = i + len(name)
        arr = u.doubles.get(name) or u.intarrs.get(name)
        if arr and j < len(e) and e[j] == "(":
            depth, k = 0, j
            while True:
                if e[k] == "(":
                    depth += 1
                elif e[k] == ")":
                    depth -= 1
                    if depth == 0:
                        break
                k += 1
            subs = [expr(x, u) for x in split_top(e[j + 1:k])]
            dims = [expr(d, u) for d in arr]
            idx = f"(({subs[-1]}) - 1)"
            for s, d in zip(reversed(subs[:-1]), reversed(dims[:-1])):
                idx = f"(({s}) - 1) + ({d}) * ({idx})"
            out += f"{name}[{idx}]"
            i = k + 1
        elif name in u.doubles and not u.doubles[name] and name in u.args:
            out += f"(*{name})"      # scalar passed by reference
            i = j
        elif getattr(u, "driver", False) and name in u.args and name not in u.intarrs:
            out += f"(*{name})"      # every scalar argument by reference
            i = j
        elif name in u.params:
            out += f"({expr(u.params[name], u)})"
            i = j
        elif u.function and name == u.name:
            out += "fret"
            i = j
        else:
            out += name
            i = j
    return out


def emit(u: Unit) -> str:
    params = []
    for a in u.args:
        if a in u.doubles:
            params.append(f"double *{a}")
        elif a in u.logicals:
            params.append(f"const int64_t *{a}_ref")
        else:
            params.append(f"const int64_t *{a}_ref")
    lines = [f"void {u.name}_({', '.join(params)}) {{"]
    for a in u.args:
        if a not in u.doubles:
            lines.append(f"  const int64_t {a} = *{a}_ref; (void){a};")
    for name in sorted(u.ints - set(u.args)):
        lines.append(f"  int64_t {name} = 0; (void){name};")
    for name, dims in u.doubles.items():
        if name in u.args:
            continue
        if dims:
            size = " * ".join(f"({expr(d, u)})" for d in dims)
            lines.append(f"  double *{name} = (double *)malloc(sizeof(double) * (size_t)({size}));")
        else:
            lines.append(f"  double {name} = 0.0; (void){name};")
    depth = 1
    for st in u.body:
        low = st.lower()
        pad = "  " * depth
        m = re.match(r"^do\s+(\w+)\s*=\s*(.+?)\s*,\s*(.+)$", st, re.I)
        if m:
            v = m.group(1).lower()
            lines.append(f"{pad}for ({v} = {expr(m.group(2), u)}; {v} <= {expr(m.group(3), u)}; {v}++) {{")
            depth += 1
            continue
        if low in ("enddo", "end do"):
            depth -= 1
            lines.append("  " * depth + "}")
            continue
        m = re.match(r"^if\s*\((.*)\)\s*then$", st, re.I)
        if m:
            lines.append(f"{pad}if ({expr(m.group(1), u)}) {{")
            depth += 1
            continue
        m = re.match(r"^else\s*if\s*\((.*)\)\s*then$", st, re.I)
        if m:
            lines.append("  " * (depth - 1) + f"}} else if ({expr(m.group(1), u)}) {{")
            continue
        if low == "else":
            lines.append("  " * (depth - 1) + "} else {")
            continue
        if low in ("endif", "end if"):
            depth -= 1
            lines.append("  " * depth + "}")
            continue
        m = re.match(r"^(.+?)\s*=\s*(.+)$", st)
        if m:
            target = m.group(1).strip().lower()
            if target in u.args and target not in u.doubles:
                raise RuntimeError(f"{u.name}: assignment to an integer argument")
            lhs = expr(m.group(1), u)
            lines.append(f"{pad}{lhs} = {expr(m.group(2), u)};")
            continue
        raise RuntimeError(f"{u.name}: statement outside the supported subset: {st}")
    for name, dims in u.doubles.items():
        if name not in u.args and dims:
            lines.append(f"  free({name});")
    lines.append("}")
    return "\n".join(lines)


def call_arg(a: str, u: Unit) -> str:
    """One actual argument of a CALL, by reference."""
    a = a.strip()
    name = a.lower()
    if re.fullmatch(r"[a-z_]\w*", name) and name not in u.params:
        if name in u.doubles and u.doubles[name] or name in u.intarrs:
            return name                          # arrays are pointers already
        if name in u.args:
            return name                          # a by-reference argument passed on
        if name in u.ints or name in u.logicals:
            return f"&{name}"
        if name in u.doubles:
            return f"&{name}"
    return f"&(int64_t){{{expr(a, u)}}}"        # an expression or a constant: a temporary


def emit_driver(u: Unit) -> str:
    """Driver-mode translation: every scalar argument by reference, integer
    arrays, labels and GOTO, CALL, RETURN; WRITE/FORMAT and timers dropped."""
    params = []
    for a in u.args:
        if a in u.doubles:
            params.append(f"double *{a}")
        else:
            params.append(f"int64_t *{a}")
    head = "int64_t" if u.function else "void"
    lines = [f"{head} {u.name}_({', '.join(params)}) {{"]
    if u.function:
        lines.append("  int64_t fret = 0;")
    for name in sorted(u.ints | u.logicals):
        if name not in u.args and name != u.name and name not in u.params:
            lines.append(f"  int64_t {name} = 0; (void){name};")
    for name, dims in u.intarrs.items():
        if name not in u.args:
            size = " * ".join(f"({int(d)})" for d in dims)
            lines.append(f"  int64_t {name}[{size}] = {{0}};")
    for name, dims in u.doubles.items():
        if name not in u.args:
            if dims:
                raise RuntimeError(f"{u.name}: local double array")
            lines.append(f"  double {name} = 0.0; (void){name};")
    ret = "return fret;" if u.function else "return;"
    depth = 1
    for st in u.body:
        label = None
        m = re.match(r"^@(\d+)\s+(.*)$", st)
        if m:
            label, st = m.group(1), m.group(2)
        low = st.lower()
        pad = "  " * depth
        if low.startswith("format"):
            continue
        if label:
            lines.append(f"{pad}L{label}:;")
        if low == "continue":
            continue
        if low.startswith("write") or "cpusecs" in low:
            continue
        m = re.match(r"^go\s*to\s+(\d+)$", st, re.I)
        if m:
            lines.append(f"{pad}goto L{m.group(1)};")
            continue
        if low == "return":
            lines.append(f"{pad}{ret}")
            continue
        m = re.match(r"^call\s+(\w+)\s*\((.*)\)$", st, re.I)
        if m:
            callee = m.group(1).lower()
            if callee == "errquit":
                lines.append(f"{pad}abort();")
            else:
                args = ", ".join(call_arg(a, u) for a in split_top(m.group(2)))
                lines.append(f"{pad}{callee}_({args});")
            continue
        m = re.match(r"^do\s+(\w+)\s*=\s*(.+)$", st, re.I)
        if m:
            v = expr(m.group(1), u)
            rng = split_top(m.group(2))
            lo, hi = expr(rng[0], u), expr(rng[1], u)
            step = expr(rng[2], u) if len(rng) > 2 else "1"
            if step.strip().startswith("-"):
                lines.append(f"{pad}for ({v} = {lo}; {v} >= {hi}; {v} += ({step})) {{")
            else:
                lines.append(f"{pad}for ({v} = {lo}; {v} <= {hi}; {v} += ({step})) {{")
            depth += 1
            continue
        if low in ("enddo", "end do"):
            depth -= 1
            lines.append("  " * depth + "}")
            continue
        m = re.match(r"^if\s*\((.*)\)\s*then$", st, re.I)
        if m:
            lines.append(f"{pad}if ({expr(m.group(1), u)}) {{")
            depth += 1
            continue
        m = re.match(r"^else\s*if\s*\((.*)\)\s*then$", st, re.I)
        if m:
            lines.append("  " * (depth - 1) + f"}} else if ({expr(m.group(1), u)}) {{")
            continue
        if low == "else":
            lines.append("  " * (depth - 1) + "} else {")
            continue
        if low in ("endif", "end if"):
            depth -= 1
            lines.append("  " * depth + "}")
            continue
        m = re.match(r"^(.+?)\s*=\s*(.+)$", st)
        if m:
            lines.append(f"{pad}{expr(m.group(1), u)} = {expr(m.group(2), u)};")
            continue
        raise RuntimeError(f"{u.name}: statement outside the supported subset: {st}")
    lines.append(f"  {ret}")
    lines.append("}")
    return "\n".join(lines)


# Fortran intrinsics and Global Arrays queries the driver sources use (one process).
DRIVER_PRELUDE = """static int64_t ieor(int64_t a, int64_t b) { return a ^ b; }
static int64_t max(int64_t a, int64_t b) { return a > b ? a : b; }
static int64_t min(int64_t a, int64_t b) { return a < b ? a : b; }
static int64_t ga_nodeid(void) { return 0; }
static int64_t ga_nnodes(void) { return 1; }
"""


def build(tree: Path = DEFAULT_TREE) -> Path:
    OUT.mkdir(exist_ok=True)
    units, drivers = [], []
    for f in FILES:
        units += parse(statements(preprocess(tree / f)))
    for f in DRIVER_FILES:
        for u in parse(statements(preprocess(tree / f)), driver=True):
            u.driver = True
            drivers.append(u)
    src = ["/* Generated by oracle/f77_ref.py from the NWChem Fortran sources; not committed. */",
           "#include <stdint.h>", "#include <stdlib.h>", ""]
    src += [emit(u) + "\n" for u in units]
    src += [DRIVER_PRELUDE]
    src += [f"{'int64_t' if u.function else 'void'} {u.name}_();" for u in drivers]   # calls between them
    src += [""] + [emit_driver(u) + "\n" for u in drivers]
    c = OUT / "ref_kernels.c"
    c.write_text("\n".join(src))
    so = OUT / "libref_kernels.so"
    res = subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11", "-o", str(so), str(c)],
                         capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(res.stderr)
    return so


if __name__ == "__main__":
    print(build(Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_TREE))
