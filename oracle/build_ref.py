"""Recipe: build the reference TensorOrder's native parts into ``oracle/_ref/``.

Test infrastructure only. Nothing in the product imports this file.

What it builds, from the sources where they lie in the reference checkout
(``TOGB_REFERENCE_ROOT``, by default a ``reference`` directory beside the
repository):

* the five Cython (C++ mode) modules listed by ``src/setup.py:4``
  (``*/*.pyx``), cythonized into ``oracle/_ref/cy`` and compiled into
  ``oracle/_ref/lib/<package>/<module>.so``;
* the FlowCutter tree-decomposition solver
  (``solvers/flow-cutter-pace17/build.sh``), compiled with ``g++`` into
  ``oracle/_ref/solvers/flow-cutter-pace17/flow_cutter_pace17`` so that the
  reference's ``util.FileLocator`` (``src/util/util.py:280-297``) finds it when
  the working directory is ``oracle/_ref``.  The shipped ``Makefile`` omits
  ``#include <string>``; ``-include string`` supplies it without editing the
  source.

Nothing is written into the reference tree.  Run ``python oracle/build_ref.py``.
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def reference_root():
    """The reference checkout: ``TOGB_REFERENCE_ROOT``, else ``../reference``
    next to this repository."""
    default = os.path.join(os.path.dirname(HERE), os.pardir, "reference")
    return os.path.normpath(os.environ.get("TOGB_REFERENCE_ROOT", default))


def flowcutter_path():
    return os.path.join(OUT, "solvers", "flow-cutter-pace17", "flow_cutter_pace17")


def build_flowcutter(force=False):
    exe = flowcutter_path()
    if os.path.exists(exe) and not force:
        return exe
    srcs = sorted(glob.glob(os.path.join(reference_root(), "solvers", "flow-cutter-pace17", "src", "*.cpp")))
    if not srcs:
        raise FileNotFoundError("FlowCutter sources not found under the reference root")
    os.makedirs(os.path.dirname(exe), exist_ok=True)
    cmd = ["g++", "-std=c++11", "-O3", "-DNDEBUG", "-include", "string", *srcs, "-o", exe]
    subprocess.check_call(cmd)
    return exe


def build_cython(force=False):
    src = os.path.join(reference_root(), "src")
    libdir = os.path.join(OUT, "lib")
    marker = os.path.join(libdir, ".built")
    if os.path.exists(marker) and not force:
        return libdir
    from Cython.Build import cythonize
    from setuptools import setup

    pyx = sorted(glob.glob(os.path.join(src, "*", "*.pyx")))
    cwd = os.getcwd()
    os.chdir(src)  # module names are derived from the package layout under src/
    try:
        exts = cythonize(
            [os.path.relpath(p, src) for p in pyx],
            language_level=3,
            build_dir=os.path.join(OUT, "cy"),
            include_path=[src],
            quiet=True,
        )
        setup(
            name="tensororder_reference_oracle",
            ext_modules=exts,
            script_args=[
                "build_ext",
                "--build-lib", libdir,
                "--build-temp", os.path.join(OUT, "tmp"),
                "-j", str(os.cpu_count() or 4),
            ],
        )
    finally:
        os.chdir(cwd)
    open(marker, "w").close()
    return libdir


def build(force=False):
    """Build both parts; returns True when the reference checkout was present."""
    if not os.path.isdir(os.path.join(reference_root(), "src")):
        return False
    build_cython(force)
    build_flowcutter(force)
    return True


if __name__ == "__main__":
    ok = build(force="--force" in sys.argv)
    print("reference oracle built" if ok else "reference checkout not present; nothing built")
