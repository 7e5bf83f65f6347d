"""Recipe that runs the reference's own Fortran on the CPU (test infrastructure).

No Fortran compiler exists on either machine, so the reference's hot-path
source files are translated to C++ by the Fortran-subset translator of this
package (``fparse``, ``funits``, ``fgen``; run-time support ``frt.h``) and
compiled with g++.  The generated source and the library go to
``oracle/_ref/`` only (kept out of version control).  Where the reference
sources are present the translation is regenerated from them; where only
the generated source is present (it travels with the repository copy) it is
compiled; otherwise nothing is built and the tests that need it skip.

The translation changes the programs in the same few places a build of the
reference on one process would (each a literal replacement of the source
text, listed in PROGRAMS):
  * ``nprocY = 8`` becomes ``nprocY = 1`` in the box program: one process,
    a single domain (the reference hard-codes 8 processes along y);
  * ``nprocY = 20`` becomes ``nprocY = 1`` in the channel program;
  * ``ipart = .false.`` becomes ``ipart = .true.`` (both programs ship with
    their particles switched off).
Problem sizes (nx, npart, rad, rhopart, ...) are module parameters in the
reference, set per build; here they are overridden at initialisation.
"""

from __future__ import annotations

import hashlib
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref"
REF_ROOT = Path(os.environ.get("LBM_REFERENCE_ROOT", "/root/reference"))

BOX_ROOTS = ["para", "allocarray", "wave", "set_plan1d_rc", "set_plan1d_cc", "initpop",
             "collision_mrt", "macrovar", "rhoupdat", "streaming", "forcing", "beads_links",
             "beads_collision", "beads_lubforce", "beads_move", "beads_redistribute",
             "beads_filling", "initpartpos", "initpartvel"]

CHANNEL_ROOTS = ["para", "allocarray", "initpop", "initvel", "collision_mrt", "macrovar",
                 "rhoupdat", "streaming", "forcing", "beads_links", "beads_collision",
                 "beads_lubforce", "beads_move", "beads_redistribute", "beads_filling",
                 "initpartpos", "initpartvel"]

PROGRAMS = {
    "box": {
        "dir": "3DBox_Forced_HI_Turbulence_Moving_Particles_LBM",
        "files": ["var_inc.f90", "para.f90", "collision.f90", "streaming.f90", "gaussian.f90",
                  "initial.f90", "partlib.f90", "mpifft.f90"],
        "patches": {"para.f90": [("nprocY = 8", "nprocY = 1"),
                                 ("ipart = .false.", "ipart = .true.")]},
        "roots": BOX_ROOTS,
    },
    "channel": {
        "dir": "3DChannel_Decaying_HIT_Finite_Size_Moving_Particles",
        "files": ["var_inc.f90", "para.f90", "collision.f90", "streaming.f90", "initial.f90",
                  "partlib.f90"],
        "patches": {"para.f90": [("nprocY = 20", "nprocY = 1"),
                                 ("ipart = .false.", "ipart = .true.")]},
        "roots": CHANNEL_ROOTS,
    },
}

CXXFLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared"]


def cpp_path(prog: str) -> Path:
    return OUT / f"ref_{prog}.cpp"


def lib_path(prog: str) -> Path:
    return OUT / f"libref_{prog}.so"


def sources_present(prog: str) -> bool:
    spec = PROGRAMS[prog]
    return all((REF_ROOT / spec["dir"] / f).exists() for f in spec["files"])


def generate(prog: str) -> Path:
    """Translate the reference's sources of `prog` into oracle/_ref/ref_<prog>.cpp."""
    sys.path.insert(0, str(HERE.parent.parent))
    from oracle.fortran.fgen import Gen
    from oracle.fortran.funits import parse_units
    spec = PROGRAMS[prog]
    units = []
    h = hashlib.sha256()
    for f in spec["files"]:
        text = (REF_ROOT / spec["dir"] / f).read_text(errors="replace")
        h.update(text.encode())
        units += parse_units(text, f, spec["patches"].get(f, ()))
    for f in ("fparse.py", "funits.py", "fgen.py"):
        h.update((HERE / f).read_bytes())
    h.update(",".join(spec["roots"]).encode())
    tag = h.hexdigest()[:16]
    out = cpp_path(prog)
    if out.exists() and f"source-hash {tag}" in out.read_text().split("\n", 2)[1]:
        return out
    src = Gen(units, f"ref_{prog}").generate(spec["roots"])
    OUT.mkdir(exist_ok=True)
    lines = src.split("\n")
    lines.insert(1, f"// source-hash {tag}")
    out.write_text("\n".join(lines))
    return out


def compile_lib(prog: str) -> Path:
    src = cpp_path(prog)
    lib = lib_path(prog)
    deps = [src, HERE / "frt.h"]
    if lib.exists() and lib.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return lib
    cmd = ["g++", *CXXFLAGS, "-I", str(HERE), str(src), "-o", str(lib)]
    subprocess.run(cmd, check=True)
    return lib


def build(prog: str = "box") -> Path | None:
    """Generate (where the reference is present) and compile; None when
    neither the reference nor a generated source is available."""
    if sources_present(prog):
        generate(prog)
    if not cpp_path(prog).exists():
        return None
    return compile_lib(prog)


def build_all() -> dict:
    return {p: build(p) for p in PROGRAMS}


if __name__ == "__main__":
    for p, lib in build_all().items():
        print(p, lib)
