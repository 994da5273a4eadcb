"""Build recipe for the checker (TEST INFRASTRUCTURE, not part of the product).

* ``build_port()`` compiles the CPU restatement in this folder into
  ``oracle/liboracle.so`` (always; it is the checker on any machine).
* ``build_ref()`` compiles the reference itself, from its sources where they lie
  under ``/root/reference`` (never copied), into ``oracle/_ref/``:
  ``libcorref.so`` (everything but the CLI) and the ``cor`` binary.  The
  environment variable COR_REFERENCE_ROOT names another location of the tree.  It is used
  only to pin the restatement and to make the golden fixtures in
  ``tests/golden/``.  It is skipped when the reference tree is absent.

Flags follow the reference's CMakeLists.txt:17 (-O3 -fno-math-errno
-fno-trapping-math -ffp-contract=off -finline-limit=300, C17, OpenMP) minus
-march=native and -Werror, so that it builds on any host.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
# where the reference tree lies (read only); COR_REFERENCE_ROOT overrides it
REF_ROOT = os.environ.get("COR_REFERENCE_ROOT", "/root/reference")
REF_OUT = os.path.join(HERE, "_ref")

FP_FLAGS = ["-O3", "-fno-math-errno", "-fno-trapping-math", "-ffp-contract=off", "-finline-limit=300"]


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + res.stdout + res.stderr)
        raise RuntimeError(f"command failed: {cmd[0]} ... {cmd[-1]}")


def _stale(out: str, srcs: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def port_sources() -> list[str]:
    return sorted(os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith(".c"))


def build_port(force: bool = False) -> str:
    out = os.path.join(HERE, "liboracle.so")
    srcs = port_sources()
    hdrs = [os.path.join(HERE, "cor_oracle.h"), os.path.join(HERE, "..", "include", "cor_trace.h")]
    if force or _stale(out, srcs + hdrs):
        objs = []
        with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
            futs = []
            for s in srcs:
                o = os.path.join(HERE, os.path.basename(s)[:-2] + ".o")
                objs.append(o)
                futs.append(ex.submit(_run, ["gcc", "-std=gnu17", "-fPIC", "-pthread", *FP_FLAGS, "-c", s, "-o", o]))
            for f in futs:
                f.result()
        _run(["gcc", "-shared", "-pthread", "-o", out, *objs, "-lm"])
        for o in objs:
            os.remove(o)
    return out


def build_nudge(force: bool = False) -> str:
    """The oracle with every libm transcendental moved by one ulp (nudge/)."""
    out = os.path.join(HERE, "liboracle_nudge.so")
    srcs = port_sources()
    nudge_dir = os.path.join(HERE, "nudge")
    extra = [os.path.join(nudge_dir, "nudge.c"), os.path.join(nudge_dir, "nudge.h")]
    if force or _stale(out, srcs + extra):
        cmd = ["gcc", "-std=gnu17", "-fPIC", "-shared", "-pthread", *FP_FLAGS, "-include",
               os.path.join(nudge_dir, "nudge.h"), *srcs, os.path.join(nudge_dir, "nudge.c"), "-o", out, "-lm"]
        _run(cmd)
    return out


def ref_available() -> bool:
    return os.path.isfile(os.path.join(REF_ROOT, "src", "trajectory.c"))


def build_ref(force: bool = False) -> str | None:
    """Compile the reference from its own sources into oracle/_ref/."""
    if not ref_available():
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    src = os.path.join(REF_ROOT, "src")
    lib = os.path.join(REF_ROOT, "lib")
    lib_srcs = [os.path.join(lib, d, f) for d in ("internal", "t96", "ts05", "chaos")
                for f in sorted(os.listdir(os.path.join(lib, d))) if f.endswith(".c")]
    core = [os.path.join(src, f) for f in ("models.c", "utils.c", "io.c", "trajectory.c", "field.c")]
    cli = [os.path.join(src, f) for f in ("main.c", "args.c")]
    so = os.path.join(REF_OUT, "libcorref.so")
    exe = os.path.join(REF_OUT, "cor")
    all_srcs = lib_srcs + core + cli
    if not force and not _stale(so, all_srcs) and not _stale(exe, all_srcs):
        return REF_OUT
    cflags = ["-std=gnu17", "-fPIC", "-fopenmp", *FP_FLAGS, f"-I{lib}", f"-I{src}"]
    objs = {}
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        futs = []
        for s in all_srcs:
            tag = os.path.relpath(s, REF_ROOT).replace(os.sep, "_")[:-2]
            o = os.path.join(REF_OUT, tag + ".o")
            objs[s] = o
            futs.append(ex.submit(_run, ["gcc", *cflags, "-c", s, "-o", o]))
        for f in futs:
            f.result()
    _run(["gcc", "-shared", "-fopenmp", "-o", so, *[objs[s] for s in lib_srcs + core], "-lm"])
    _run(["gcc", "-fopenmp", "-o", exe, *[objs[s] for s in lib_srcs + core + cli], "-lm"])
    for o in objs.values():
        os.remove(o)
    return REF_OUT


def build_shim(force: bool = False) -> str | None:
    """The reference's own `cor` program with its trajectory_simulation_cutoff
    replaced by cor-model_gb300/host/trajectory_shim.c and linked against
    libcortrace.so, into oracle/_ref/cor_shim: the link-in drop-in a
    maintainer would build.  The reference's definition in src/trajectory.c is
    renamed away at compile time; everything else of the reference (main,
    argument parsing, INFILE reader, model registry and set-up, output
    header) is its own code.  Needs the reference tree and the built library;
    returns None without them."""
    pkg = os.path.join(HERE, "..", "cor-model_gb300")
    lib_so = os.path.join(pkg, "libcortrace.so")
    if not ref_available() or not os.path.exists(lib_so):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    src = os.path.join(REF_ROOT, "src")
    lib = os.path.join(REF_ROOT, "lib")
    lib_srcs = [os.path.join(lib, d, f) for d in ("internal", "t96", "ts05", "chaos")
                for f in sorted(os.listdir(os.path.join(lib, d))) if f.endswith(".c")]
    ref_srcs = lib_srcs + [os.path.join(src, f) for f in ("models.c", "utils.c", "io.c", "field.c", "trajectory.c",
                                                         "main.c", "args.c")]
    shim = os.path.join(pkg, "host", "trajectory_shim.c")
    exe = os.path.join(REF_OUT, "cor_shim")
    deps = ref_srcs + [shim, os.path.join(pkg, "host", "scan_text.h"), lib_so]
    if not force and not _stale(exe, deps):
        return exe
    cflags = ["-std=gnu17", "-fopenmp", *FP_FLAGS, f"-I{lib}", f"-I{src}"]
    objs = []
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        futs = []
        for s in ref_srcs:
            o = os.path.join(REF_OUT, "shim_" + os.path.relpath(s, REF_ROOT).replace(os.sep, "_")[:-2] + ".o")
            extra = ["-Dtrajectory_simulation_cutoff=reference_trajectory_simulation_cutoff_replaced"] \
                if s.endswith("trajectory.c") else []
            objs.append(o)
            futs.append(ex.submit(_run, ["gcc", *cflags, *extra, "-c", s, "-o", o]))
        o = os.path.join(REF_OUT, "shim_trajectory_shim.o")
        objs.append(o)
        futs.append(ex.submit(_run, ["gcc", *cflags, f"-I{os.path.join(HERE, '..', 'include')}",
                                     f"-I{os.path.join(pkg, 'host')}", "-c", shim, "-o", o]))
        for f in futs:
            f.result()
    _run(["gcc", "-fopenmp", "-o", exe, *objs, f"-L{pkg}", "-lcortrace", f"-Wl,-rpath,{os.path.abspath(pkg)}",
          "-lm"])
    for o in objs:
        os.remove(o)
    return exe


if __name__ == "__main__":
    print(build_port(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
