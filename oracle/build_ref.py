#!/usr/bin/env python3
"""Recipe that compiles the reference itself, headlessly, into oracle/_ref/.

Test infrastructure only.  Steps:

1. ``snapshot``: when a reference checkout is named (``--ref-dir DIR`` or the
   REF_DIR environment variable), copy the C files its wave path is built from into
   oracle/_ref/src/.  Without one, the existing snapshot is compiled.  oracle/_ref/ is git-ignored (never committed) but travels with
   the working tree, so a machine without the checkout can still compile it.
2. ``generate``: for every configuration in oracle/ref_variants.py, write a
   translation unit into oracle/_ref/src/gen/ whose ``#define`` values are the
   variant's.  Full builds take the whole program; function builds take the define
   block, global_pdes.c and the hot-path functions cut verbatim out of the
   reference files by name.  One patch is applied to evolve_wave_half: the corner
   write ``phi_out[0][NX-1] = oscillating_bc(time, NX-1);`` (wave_billiard.c:589),
   which lands outside row 0 when NX > NY, is guarded by ``if (NX <= NY)``.
3. ``compile``: gcc -O2 -fopenmp -ffp-contract=off (no FMA contraction, no -march)
   of oracle/ref_driver.c around each unit, in parallel, into oracle/_ref/bin/.
   Variants marked ``stock`` use the reference makefile's own flags instead
   (gcc -O3 -fopenmp, the compiler's default contraction): those are timed as the CPU
   baseline, never used for parity.
   The ``*__dropin`` variants are the same units with the reference's evolve_wave /
   evolve_wave_half replaced by include/wavegpu_dropin.h, linked to libwavegpu.so:
   the reference's own driver code stepping on the GPU (built once the library
   exists).

Usage: python oracle/build_ref.py [--ref-dir DIR] [--only NAME ...] [--jobs N]
"""
import argparse
import hashlib
import os
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import ref_variants  # noqa: E402

REF_DIR = Path(os.environ["REF_DIR"]) if os.environ.get("REF_DIR") else None
OUT = HERE / "_ref"
SRC = OUT / "src"
GEN = SRC / "gen"
BIN = OUT / "bin"
STUBS = HERE / "stubs"
INCLUDE = HERE.parent / "include"
LIBDIR = HERE.parent / "youtube-simulations_gb300"

SOURCES = ["wave_billiard.c", "wave_energy.c", "global_pdes.c", "sub_maze.c", "sub_wave.c",
           "wave_common.c", "sub_wave_comp.c", "colors_waves.c", "colormaps.c",
           "turbo_colormap.c", "hsluv.c", "hsluv.h"]

Q2_FROM = "phi_out[0][NX-1] = oscillating_bc(time, NX-1);"
Q2_TO = "if (NX <= NY) phi_out[0][NX-1] = oscillating_bc(time, NX-1);"


def snapshot(ref_dir=None):
    """Copy the reference sources from the checkout `ref_dir` into oracle/_ref/src."""
    ref_dir = Path(ref_dir) if ref_dir else REF_DIR
    if ref_dir is None or not ref_dir.is_dir():
        return False
    SRC.mkdir(parents=True, exist_ok=True)
    manifest = []
    for name in SOURCES:
        data = (ref_dir / name).read_bytes()
        dst = SRC / name
        if not dst.exists() or dst.read_bytes() != data:
            dst.write_bytes(data)
        manifest.append(f"{hashlib.sha256(data).hexdigest()}  {name}")
    (SRC / "MANIFEST.sha256").write_text("\n".join(manifest) + "\n")
    return True


def _read(name):
    return (SRC / name).read_text(encoding="latin-1")


def define_block(prog_text):
    """Everything before the program's `#include "global_pdes.c"` line."""
    idx = prog_text.index('#include "global_pdes.c"')
    return prog_text[:idx]


def patch_defines(text, macros):
    """Set each macro's value in a define block; append the ones it lacks."""
    done = set()
    out = []
    for line in text.split("\n"):
        m = re.match(r"^(\s*#define\s+)([A-Za-z_][A-Za-z0-9_]*)(\s+)(\S+)(.*)$", line)
        if m and m.group(2) in macros and m.group(2) not in done:
            name = m.group(2)
            line = f"{m.group(1)}{name}{m.group(3)}{ref_variants.macro_text(macros[name])}{m.group(5)}"
            done.add(name)
        out.append(line)
    missing = [k for k in macros if k not in done]
    # A define that the program lacks is appended; one that it defines twice keeps
    # its first occurrence patched and later redefinitions are dropped by #undef.
    extra = [f"#undef {k}\n#define {k} {ref_variants.macro_text(macros[k])}" for k in missing]
    return "\n".join(out) + "\n" + "\n".join(extra) + "\n"


def extract_function(text, name):
    """Cut a top-level C function definition (signature through closing brace)."""
    m = re.search(r"^[A-Za-z_][A-Za-z0-9_ \*]*\b" + re.escape(name) + r"\s*\([^;{]*?\)\s*(/\*.*?\*/\s*)*\{",
                  text, re.M | re.S)
    if not m:
        raise KeyError(name)
    depth = 0
    i = text.index("{", m.end() - 1)
    j = i
    while True:
        c = text[j]
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                return text[m.start():j + 1] + "\n"
        elif c == "/" and text[j + 1] == "*":
            j = text.index("*/", j + 2) + 1
        elif c == "/" and text[j + 1] == "/":
            j = text.index("\n", j)
        j += 1


def generate(name, spec):
    kind, macros = spec["kind"], spec["macros"]
    GEN.mkdir(parents=True, exist_ok=True)
    if kind == "wb_full":
        prog = _read("wave_billiard.c")
        blk = define_block(prog)
        body = prog[len(blk):]
        assert Q2_FROM in body
        text = patch_defines(blk, macros) + body.replace(Q2_FROM, Q2_TO)
    else:
        prog_name = "wave_energy.c" if kind == "we_fn" else "wave_billiard.c"
        prog = _read(prog_name)
        sub = _read("sub_wave.c")
        common = _read("wave_common.c")
        parts = [patch_defines(define_block(prog), macros), '#include "global_pdes.c"\n',
                 "double vabs(double x);\n",
                 extract_function(sub, "xy_to_ij"), extract_function(sub, "oscillating_bc")]
        if kind == "wb_fn" and spec.get("dropin"):
            # the reference with its stepper replaced by the GPU drop-in header
            parts += [extract_function(common, "compute_energy"), '#include "wavegpu_dropin.h"\n']
        elif kind == "wb_fn":
            parts += [extract_function(common, "compute_energy"),
                      extract_function(prog, "evolve_wave_half").replace(Q2_FROM, Q2_TO),
                      extract_function(prog, "evolve_wave")]
        elif kind == "we_fn":
            comp = _read("sub_wave_comp.c")
            parts += ["double courant2, courantb2;\n",
                      extract_function(common, "compute_energy"),
                      extract_function(prog, "compute_energy_x"),
                      extract_function(comp, "compute_energy_tblr"),
                      extract_function(prog, "evolve_wave_half"),
                      extract_function(prog, "evolve_wave")]
        text = "".join(parts)
    path = GEN / f"{name}.c"
    if not path.exists() or path.read_text(encoding="latin-1") != text:
        path.write_text(text, encoding="latin-1")
    return path


def compile_one(name, spec, cc="gcc"):
    BIN.mkdir(parents=True, exist_ok=True)
    kind = spec["kind"]
    tu = GEN / f"{name}.c"
    exe = BIN / f"ref_{name}"
    defs = {"wb_full": ["-DREF_KIND_WB", "-DREF_FULL"], "wb_fn": ["-DREF_KIND_WB"],
            "we_fn": ["-DREF_KIND_WE"], "osc": ["-DREF_KIND_OSC"]}[kind]
    opt = ["-O3", "-fopenmp"] if spec.get("stock") else ["-O2", "-fopenmp", "-ffp-contract=off"]
    cmd = [cc, *opt, "-w", "-std=gnu99",
           f"-I{STUBS}", f"-I{SRC}", f"-I{GEN}", f'-DREF_TU="{tu.name}"', *defs,
           str(HERE / "ref_driver.c"), "-o", str(exe), "-lm"]
    if spec.get("dropin"):
        cmd += [f"-I{INCLUDE}", f"-L{LIBDIR}", "-lwavegpu", f"-Wl,-rpath,{LIBDIR}"]
    deps = [tu, HERE / "ref_driver.c"] + ([LIBDIR / "libwavegpu.so", INCLUDE / "wavegpu_dropin.h"]
                                          if spec.get("dropin") else [])
    if exe.exists() and exe.stat().st_mtime > max(d.stat().st_mtime for d in deps):
        return name, 0, ""
    r = subprocess.run(cmd, capture_output=True, text=True)
    return name, r.returncode, r.stderr[-2000:]


def available():
    return (SRC / "wave_billiard.c").exists()


def build(only=None, jobs=None, ref_dir=None):
    snapshot(ref_dir)
    if not available():
        print("build_ref: reference sources not present; skipping", file=sys.stderr)
        return False
    names = only or list(ref_variants.VARIANTS)
    # drop-in builds need the GPU library (built first by the package's build)
    if not (LIBDIR / "libwavegpu.so").exists():
        names = [n for n in names if not ref_variants.VARIANTS[n].get("dropin")]
    for n in names:
        generate(n, ref_variants.VARIANTS[n])
    jobs = jobs or os.cpu_count() or 4
    ok = True
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        for name, rc, err in ex.map(lambda n: compile_one(n, ref_variants.VARIANTS[n]), names):
            if rc != 0:
                ok = False
                print(f"build_ref: {name} failed:\n{err}", file=sys.stderr)
    return ok


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-dir", help="reference checkout to snapshot from (default: $REF_DIR)")
    ap.add_argument("--only", nargs="*")
    ap.add_argument("--jobs", type=int)
    a = ap.parse_args()
    sys.exit(0 if build(a.only, a.jobs, a.ref_dir) else 1)
