"""Builds the test-only frontier operators of tests/plugins/ against libmg
(nvcc for sm_103a, as include/mg_plugin.cuh describes) into
tests/plugins/_build/.  Used by the plugin tests."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "multigraph_gb300")


def build_plugin(name: str) -> str:
    from multigraph_gb300 import build as b
    b.build()
    src = os.path.join(HERE, "plugins", name + ".cu")
    out_dir = os.path.join(HERE, "plugins", "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "lib" + name + ".so")
    deps = [src, os.path.join(PKG, "libmg.so")] + [
        os.path.join(d, f) for d in (os.path.join(ROOT, "include"), os.path.join(PKG, "csrc"))
        for f in os.listdir(d) if f.endswith((".h", ".cuh"))]
    if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(d) for d in deps):
        return out
    cmd = [b._nvcc(), b.GENCODE, "-std=c++17", "-O3", "-shared", "-Xcompiler", "-fPIC",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(PKG, "csrc"), src,
           "-L", PKG, "-lmg", "-Xlinker", "-rpath=" + PKG, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("plugin build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return out
