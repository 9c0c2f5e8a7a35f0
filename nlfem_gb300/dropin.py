"""Builds the reference's own Python module against this library: the drop-in recipe.

The reference's cython/nlfem.pyx binds its C++ through include/Cassemble.pxd
(`cdef extern from "Cassemble.h"`). This library ships a header of that name
(include/Cassemble.h, which includes Cassemble_compat.h) and exports the same C++ symbols from
libnlfem_gpu.so (par_assemble, par_evaluateMass, method_retriangulate,
method_retriangulateInfty, toRef, toPhys, solve2x2). So the unchanged .pyx compiles and links
against it:

    from nlfem_gb300 import dropin
    cpp = dropin.generate("<reference checkout>")          # needs Cython; C++ into GENERATED
    so = dropin.compile_module(cpp, "<build dir>")         # needs g++ and Python's headers
    # then: sys.path.insert(0, "<build dir>"); import nlfem

Steps: cythonize <reference>/cython/nlfem.pyx (read in place; the generated C++ goes to
nlfem_gb300/_dropin/), with <reference>/include on Cython's include path for Cassemble.pxd; compile
the generated C++ with this library's include/ first on the compiler's include path; link against
libnlfem_gpu.so (rpath set). Nothing of the reference is modified or copied.

The reference's module still calls numpy's removed alias np.int (nlfem.pyx:394, 427 and the zeta
branches); on numpy >= 1.24 a caller sets `numpy.int = int` before using those functions.
"""
import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# Where generate() leaves the generated C++ by default (git-ignored). The two halves can run on
# different machines: cythonize where Cython and the reference checkout are, compile where the GPU is.
GENERATED = os.path.join(HERE, "_dropin")
GENERATED_CPP = os.path.join(GENERATED, "nlfem.cpp")


def generate(reference, out_dir=GENERATED):
    """Cythonize the reference's nlfem.pyx; returns out_dir/nlfem.cpp. Skips the work when that
    file is newer than the .pyx and the .pxd."""
    import shutil
    import tempfile
    ref = os.path.abspath(reference)
    pyx = os.path.join(ref, "cython", "nlfem.pyx")
    pxd = os.path.join(ref, "include", "Cassemble.pxd")
    if not os.path.exists(pyx):
        raise FileNotFoundError(pyx)
    os.makedirs(out_dir, exist_ok=True)
    dst = os.path.join(out_dir, "nlfem.cpp")
    if os.path.exists(dst) and os.path.getmtime(dst) > max(os.path.getmtime(pyx), os.path.getmtime(pxd)):
        return dst
    from Cython.Build import cythonize
    with tempfile.TemporaryDirectory() as tmp:
        cythonize([pyx], include_path=[os.path.join(ref, "include")], language="c++", build_dir=tmp,
                  quiet=True, compiler_directives={"language_level": 3})
        for dirpath, _, files in os.walk(tmp):
            if "nlfem.cpp" in files:
                shutil.copyfile(os.path.join(dirpath, "nlfem.cpp"), dst + ".tmp")
                os.replace(dst + ".tmp", dst)
                return dst
    raise RuntimeError("cythonize produced no nlfem.cpp")


def can_compile():
    """True when Python's headers (Python.h) are present, which compile_module needs."""
    return os.path.exists(os.path.join(sysconfig.get_paths()["include"], "Python.h"))


def compile_module(cpp, out_dir):
    """Compile a generated nlfem.cpp into the extension module nlfem<EXT_SUFFIX> in out_dir,
    against include/ and libnlfem_gpu.so of this package."""
    import numpy
    from . import build
    lib = build.build()
    os.makedirs(out_dir, exist_ok=True)
    so = os.path.join(os.path.abspath(out_dir), "nlfem" + sysconfig.get_config_var("EXT_SUFFIX"))
    cmd = ["g++", "-O2", "-shared", "-fPIC", "-std=c++17", "-w", cpp, "-o", so,
           "-I" + os.path.join(ROOT, "include"), "-I" + numpy.get_include(), "-I" + sysconfig.get_paths()["include"],
           "-L" + os.path.dirname(lib), "-l:" + os.path.basename(lib), "-Wl,-rpath," + os.path.dirname(lib)]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("compiling the reference module failed:\n" + p.stderr[-4000:])
    return so


def build_reference_module(reference, out_dir):
    """generate + compile_module; returns the path of the built extension module."""
    return compile_module(generate(reference), out_dir)


if __name__ == "__main__":
    if len(sys.argv) != 3:
        raise SystemExit("usage: python -m nlfem_gb300.dropin <reference checkout> <build dir>")
    print(build_reference_module(sys.argv[1], sys.argv[2]))
