"""Build the reference harness (TEST INFRASTRUCTURE ONLY).

Where the read-only reference tree is present (the development container),
its `src/` and `inc/` directories are staged into oracle/_ref/ so that the
reference can be compiled on a machine without that tree (the GPU host).
oracle/_ref/ is git-ignored: the staged files and the binary are build
inputs/outputs, never part of the repository.  Wherever oracle/_ref/src
exists and nvcc is available, oracle/ref_harness.cu is compiled against it
into oracle/_ref/ref_harness (sm_103a, the reference sources unmodified;
oracle/ref_shim.h is force-included to restore cub::Max, which CUDA 13's
CCCL removed).
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
# the read-only reference checkout; HSMU_REFERENCE_TREE names another location
REF_TREE = os.environ.get("HSMU_REFERENCE_TREE", "/root/reference")
OUT = os.path.join(HERE, "_ref")
BIN = os.path.join(OUT, "ref_harness")


def stage() -> bool:
    """Copy the reference's src/ and inc/ into oracle/_ref/ (if the tree exists)."""
    if not os.path.isdir(os.path.join(REF_TREE, "src")):
        return False
    os.makedirs(OUT, exist_ok=True)
    for d in ("src", "inc"):
        dst = os.path.join(OUT, d)
        if os.path.isdir(dst):
            shutil.rmtree(dst)
        shutil.copytree(os.path.join(REF_TREE, d), dst,
                        ignore=shutil.ignore_patterns("*.o", "*.bin", "a.out"))
        for root, dirs, files in os.walk(dst):
            for n in dirs:
                os.chmod(os.path.join(root, n), 0o755)
            for n in files:
                os.chmod(os.path.join(root, n), 0o644)
        os.chmod(dst, 0o755)
    return True


def build(force: bool = False) -> str | None:
    """Compile the harness if the staged sources exist; returns the binary path."""
    if not os.path.isdir(os.path.join(OUT, "src")):
        return None
    src = os.path.join(HERE, "ref_harness.cu")
    if not force and os.path.exists(BIN) and os.path.getmtime(BIN) >= os.path.getmtime(src):
        try:
            with open(BIN, "rb") as f:
                magic = f.read(20)
            import platform

            machine = {"x86_64": 62, "aarch64": 183}.get(platform.machine())
            if magic[:4] == b"\x7fELF" and (machine is None or int.from_bytes(magic[18:20], "little") == machine):
                return BIN
        except OSError:
            pass
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    if not os.path.exists(nvcc):
        nvcc = "nvcc"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-w",
           "-include", os.path.join(HERE, "ref_shim.h"), "-I", OUT, src, "-o", BIN + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference harness build failed:\n" + r.stderr[-4000:])
    os.replace(BIN + ".tmp", BIN)
    return BIN


def build_if_present() -> str | None:
    stage()
    return build()


if __name__ == "__main__":
    print(build_if_present())
