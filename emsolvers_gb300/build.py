"""Builds libems.so (C++ host + sm_103a CUDA kernels) in-tree with nvcc.

Every translation unit is compiled in parallel for sm_103a only, then linked
into emsolvers_gb300/_build/libems.so together with the ems_fem command-line
driver.  Static cudart, so the library needs nothing but the driver at run
time.  `python -m emsolvers_gb300.build` rebuilds.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libems.so")
CLI = os.path.join(OUT, "ems_fem")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")) and not f.startswith("cli_"))


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off", "--expt-relaxed-constexpr",
                   "-I" + os.path.join(ROOT, "include")]


def _up_to_date(target, deps):
    return os.path.exists(target) and all(os.path.getmtime(target) >= os.path.getmtime(d) for d in deps)


def build(force=False, verbose=False, ptxas_info=False):
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "ems.h"))
    jobs = []
    objs = []
    for src in _sources():
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or not _up_to_date(o, [s] + headers):
            cmd = [cc] + _flags() + ["-c", s, "-o", o + ".tmp"]
            if ptxas_info and src.endswith(".cu"):
                cmd += ["-Xptxas", "-v"]
            jobs.append((cmd, o))

    def run(job):
        cmd, o = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        os.replace(o + ".tmp", o)
        return r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for log in ex.map(run, jobs):
            if verbose and log.strip():
                print(log)
    if force or jobs or not os.path.exists(LIB):
        cmd = [cc] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    cli_src = os.path.join(CSRC, "cli_fem.cpp")
    if os.path.exists(cli_src) and (force or not _up_to_date(CLI, [cli_src, LIB])):
        cmd = [cc] + _flags() + [cli_src, "-o", CLI, "-L" + OUT, "-lems", "-Xlinker", "-rpath,$ORIGIN"]
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
