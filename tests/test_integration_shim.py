"""The C shim a maintainer drops in place of src/qubatron/octree_glc.c
(include/examples/octree_cuda.c: octree_glc_* on top of libqbcuda)
compiles against include/qbcuda.h and links against the built library. No
GPU."""
import os
import subprocess

from conftest import ROOT


def test_shim_compiles_and_links(lib, tmp_path):
    src = os.path.join(ROOT, "include", "examples", "octree_cuda.c")
    # the reference tree provides v3_t in src/mt_math/mt_vector_3d.c; a
    # stand-in with the same layout for compiling outside it
    stub = tmp_path / "stub"
    stub.mkdir()
    (stub / "mt_vector_3d.c").write_text("typedef struct _v3_t { float x, y, z; } v3_t;\n")
    lib_dir = os.path.join(ROOT, "qubatron_gb300", "_build")
    subprocess.run(["gcc", "-std=c99", "-fPIC", "-Wall", "-Werror", "-Wno-unused-function", "-c",
                    "-I", str(stub), "-I", os.path.join(ROOT, "include"), src, "-o", str(tmp_path / "shim.o")],
                   check=True)
    subprocess.run(["gcc", "-shared", "-o", str(tmp_path / "liboctree_cuda.so"), str(tmp_path / "shim.o"),
                    f"-L{lib_dir}", "-lqbcuda", f"-Wl,-rpath,{lib_dir}"], check=True)
