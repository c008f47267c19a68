"""Build libControllerEngine.so in-tree (nvcc for sm_103a, g++ for host code).

Translation units compile in parallel; the library is written to
controllerengine_gb300/_lib/libControllerEngine.so.  Host code is built with
-ffp-contract=off so that no multiply-add is fused on any host architecture
(GCC fuses by default on aarch64); device code controls fusion with explicit
round-to-nearest intrinsics.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
LIB = OUT / "libControllerEngine.so"
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["ce_k_sim.cu", "ce_k_eig.cu", "ce_k_modal.cu", "ce_k_sweep.cu", "ce_k_calib.cu", "ce_noalloc.cu", "ce_k_plant.cu",
              "ce_k_kalman.cu"]
CPP_SOURCES = ["ce_config.cpp", "ce_engine.cpp", "ce_jit.cpp", "ce_server.cpp"]
# headers the run-time specialiser (ce_jit.cpp) hands to NVRTC, by the name they are #included under
JIT_HEADERS = [("ce_sim_body.cuh", "ce_sim_body.cuh"), ("ce_device.cuh", "ce_device.cuh"),
               ("ce_internal.h", "ce_internal.h"), ("../../include/controller_engine.h", None)]


def _run(cmd: list[str]) -> str:
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"command failed ({p.returncode}): {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
    return p.stdout + p.stderr


def _digest() -> str:
    h = hashlib.sha256()
    for f in sorted(CSRC.iterdir()):
        if f.suffix in (".cu", ".cuh", ".cpp", ".h"):
            h.update(f.name.encode())
            h.update(f.read_bytes())
    h.update((ROOT / "include" / "controller_engine.h").read_bytes())
    h.update(Path(__file__).read_bytes())
    return h.hexdigest()[:16]


def _write_jit_headers(path: Path):
    parts = ["// generated by controllerengine_gb300/build.py: headers compiled by NVRTC at run time",
             "struct JitHeader { const char* name; const char* text; };",
             "const JitHeader kJitHeaders[] = {"]
    for name, rel in JIT_HEADERS:
        src = (CSRC / rel) if rel else (ROOT / "include" / "controller_engine.h")
        text = src.read_text()
        assert ")CE_SRC\"" not in text
        parts.append(f'    {{"{name}", R"CE_SRC({text})CE_SRC"}},')
    parts.append("};")
    path.write_text("\n".join(parts) + "\n")


def build(verbose: bool = False, ptxas_info: bool = False, force: bool = False) -> Path:
    """Compile and link the library; returns its path.  Skips work if sources are unchanged."""
    OUT.mkdir(exist_ok=True)
    stamp = OUT / "build.stamp"
    dig = _digest()
    if not force and LIB.exists() and stamp.exists() and stamp.read_text().strip() == dig:
        return LIB
    objdir = OUT / "obj"
    if objdir.exists():
        shutil.rmtree(objdir)
    objdir.mkdir()
    gen = OUT / "gen"
    gen.mkdir(exist_ok=True)
    _write_jit_headers(gen / "ce_jit_src.inc")
    inc = ["-I", str(ROOT / "include"), "-I", str(CSRC), "-I", str(gen)]
    jobs = []
    for src in CU_SOURCES:
        obj = objdir / (src + ".o")
        cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++20", "--expt-relaxed-constexpr",
               "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden", *inc, "-c", str(CSRC / src), "-o", str(obj)]
        if ptxas_info:
            cmd += ["-Xptxas", "-v"]
        jobs.append(cmd)
    for src in CPP_SOURCES:
        obj = objdir / (src + ".o")
        cmd = ["g++", "-O2", "-std=c++20", "-fPIC", "-ffp-contract=off", "-fvisibility=hidden",
               f'-DCE_CUDA_INCLUDE="{CUDA_HOME / "include"}"',
               "-I", str(CUDA_HOME / "include"), *inc, "-c", str(CSRC / src), "-o", str(obj)]
        jobs.append(cmd)
    logs = []
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    objs = [str(objdir / (s + ".o")) for s in CU_SOURCES + CPP_SOURCES]
    tmp = OUT / (LIB.name + ".tmp")
    _run([NVCC, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *objs,
          "-L", str(CUDA_HOME / "lib64"), "-lnvrtc", f"-Xlinker=-rpath,{CUDA_HOME / 'lib64'}",
          "-lpthread", "-ldl", "-lrt"])
    os.replace(tmp, LIB)
    stamp.write_text(dig)
    if verbose or ptxas_info:
        sys.stdout.write("\n".join(l for l in logs if l.strip()) + "\n")
    return LIB


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv, force=force))
