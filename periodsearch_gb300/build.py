"""Builds the engine in-tree: libps_gb300.so (C ABI) and the ps_gb300 CLI.

The translation units are compiled in parallel: the sm_103a kernels with
nvcc, the host code with g++ (-ffp-contract=off keeps the reference's
rounding in the per-object set-up on FMA hosts such as aarch64).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = ROOT / "_build"
LIB = PKG / "libps_gb300.so"
CLI = PKG / "ps_gb300"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> Path:
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError(f"build step failed: {cmd[0]} {cmd[-1]}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    inc = ["-I", str(ROOT / "include"), "-I", str(CSRC)]
    BUILD.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "ps_gb300.h"]
    units = {
        "ps_engine.o": [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                        "-Xptxas", "-v" if verbose else "-O3", *inc,
                        "-c", str(CSRC / "ps_engine.cu"), "-o", str(BUILD / "ps_engine.o")],
        "ps_mlp.o": [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", *inc,
                     "-c", str(CSRC / "ps_mlp.cu"), "-o", str(BUILD / "ps_mlp.o")],
        "ps_tc.o": [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", *inc,
                    "-c", str(CSRC / "ps_tc.cu"), "-o", str(BUILD / "ps_tc.o")],
        "ps_pack.o": [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", *inc,
                      "-c", str(CSRC / "ps_pack.cu"), "-o", str(BUILD / "ps_pack.o")],
        "ps_api.o": ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", *inc,
                     "-I", str(cuda / "include"), "-c", str(CSRC / "ps_api.cpp"), "-o", str(BUILD / "ps_api.o")],
        "ps_setup.o": ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", *inc,
                       "-c", str(CSRC / "ps_setup.cpp"), "-o", str(BUILD / "ps_setup.o")],
        "ps_validate.o": ["g++", "-O2", "-std=c++17", "-fPIC", *inc,
                          "-c", str(CSRC / "ps_validate.cpp"), "-o", str(BUILD / "ps_validate.o")],
    }
    srcs = {"ps_engine.o": CSRC / "ps_engine.cu", "ps_mlp.o": CSRC / "ps_mlp.cu", "ps_api.o": CSRC / "ps_api.cpp",
            "ps_setup.o": CSRC / "ps_setup.cpp", "ps_validate.o": CSRC / "ps_validate.cpp", "ps_tc.o": CSRC / "ps_tc.cu",
            "ps_pack.o": CSRC / "ps_pack.cu"}
    todo = [cmd for obj, cmd in units.items() if force or _stale(BUILD / obj, [srcs[obj], *headers])]
    with ThreadPoolExecutor(max_workers=8) as ex:
        list(ex.map(_run, todo))
    objs = [str(BUILD / o) for o in units]
    if force or todo or _stale(LIB, [Path(o) for o in objs]):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *objs, "-lcudart"])
    if force or _stale(CLI, [LIB, CSRC / "ps_cli.cpp"]):
        _run(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "include"), str(CSRC / "ps_cli.cpp"), "-o", str(CLI),
              "-L", str(PKG), "-lps_gb300", f"-Wl,-rpath,{PKG}", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
