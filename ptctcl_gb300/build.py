"""Build libhora_gb300.so for sm_103a with nvcc, in-tree (ptctcl_gb300/_build/).

Every kernel is a template on the DBM dimension D (clocks + 1). Two translation units per D in
[1, 17] are generated and compiled in parallel, then linked with the host/C-ABI unit into one
shared library whose exported surface is exactly include/hora_gb300.h.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
GEN = os.path.join(BUILD, "gen")
LIB = os.path.join(BUILD, "libhora_gb300.so")
DIMS = list(range(1, 18))
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "--expt-relaxed-constexpr", "-Xptxas", "-O3", *ARCH]

# Two units per dimension, compiled in parallel: the level kernels with the engine, and the
# subsumed leads-to graph with its federation sweep (whose members are instantiated there; the class
# instantiation of the first unit covers only the members it defines).
SUB_UNIT = """// generated by ptctcl_gb300/build.py: subsumed leads-to kernels for DBM dimension {D}
#include "../../csrc/level_kernels_impl.cuh"
#include "../../csrc/subsumed_impl.cuh"
namespace hgb {{
template void Level<{D}>::incl_probe(const NetView*, InstState, Succ, Store, Ctl*, long long, int, cudaStream_t);
template void Level<{D}>::incl_group(Succ, Store, Ctl*, long long, long long, cudaStream_t);
template void Level<{D}>::incl_keep(Succ, Store, Ctl*, long long, int, cudaStream_t);
template void Level<{D}>::incl_store(const NetView*, InstState, Succ, Store, Front, Ctl*, long long, int, int,
                                     cudaStream_t);
template void Level<{D}>::incl_lists(const NetView*, InstState, Succ, Store, Ctl*, long long, cudaStream_t);
template void Level<{D}>::incl_cover(Succ, Store, Ctl*, long long, int, cudaStream_t);
template void Level<{D}>::incl_edges(Succ, Front, Edges, Ctl*, long long, cudaStream_t);
template void Level<{D}>::stop_fed(const NetView*, InstState, Store, long long, long long, const int*, Fix, Ctl*, int,
                                   int, cudaStream_t);
template void Level<{D}>::edge_csr(Edges, long long, long long, int*, int*, int*, cudaStream_t);
template void Level<{D}>::gfp_init(Fix, long long, Ctl*, cudaStream_t);
template void Level<{D}>::gfp_relax(const NetView*, Store, Edges, Fix, Ctl*, long long, int, cudaStream_t);
template void Level<{D}>::gfp_round_end(Edges, long long, long long, Fix, const int*, Ctl*, cudaStream_t);
template void Level<{D}>::gfp_compact(Fix, long long, int*, unsigned long long*, cudaStream_t);
template void Level<{D}>::gfp_verdict_fed(const NetView*, Store, long long, Fix, InstState, cudaStream_t);
template long long Level<{D}>::relax_tiles(int);
}}  // namespace hgb
"""

DIM_UNIT = """// generated by ptctcl_gb300/build.py: instantiations for DBM dimension {D}
#include "../../csrc/level_kernels_impl.cuh"
#include "../../csrc/engine_run.cuh"
namespace hgb {{
template struct Level<{D}>;
template int run_group<{D}>(const std::vector<const HostNet*>&, std::vector<InstResult>&, const RunOptions&,
                            std::string&);
template int run_expand<{D}>(const HostNet&, int, const int*, const int*, const int*, int, int64_t, int*, int*,
                             int*, int*, int*, int64_t*, std::string&);
template int run_has_deadlock<{D}>(const HostNet&, int, const int*, const int*, const int*, int*, std::string&);
}}  // namespace hgb
"""


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h"))] + \
        [os.path.join(HERE, "..", "include", "hora_gb300.h"), os.path.abspath(__file__)]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(GEN, exist_ok=True)
    units = []
    for d in reversed(DIMS):   # the largest dimensions compile longest: start them first
        for name, text in ((f"dim_{d}.cu", DIM_UNIT), (f"sub_{d}.cu", SUB_UNIT)):
            p = os.path.join(GEN, name)
            src = text.format(D=d)
            if not os.path.exists(p) or open(p).read() != src:
                with open(p, "w") as fh:
                    fh.write(src)
            units.append(p)
    units.append(os.path.join(CSRC, "host.cu"))
    units += [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith(".cu") and f != "host.cu"]
    cc = nvcc()
    objs = []

    def compile_one(u):
        o = os.path.join(BUILD, os.path.basename(u).replace(".cu", ".o"))
        out = _run([cc, *NVCC_FLAGS, "-c", u, "-o", o] + (["-Xptxas", "-v"] if verbose else []))
        return o, out

    jobs = jobs or min(len(units), max(2, os.cpu_count() or 4))
    with ThreadPoolExecutor(jobs) as ex:
        for o, out in ex.map(compile_one, units):
            objs.append(o)
            if verbose and out:
                sys.stderr.write(out)
    tmp = LIB + ".tmp"
    _run([cc, *ARCH, "-shared", "-cudart=static", "-o", tmp, *objs])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
