"""Build recipe for ``oracle/_ref``: the reference's own Cython modules, compiled as a checker.

This is test infrastructure.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` use what it builds, and only as the thing the
CUDA path is checked against or timed beside.

Two stages:

``generate`` (needs Cython and the reference tree; runs where the reference is
mounted).  Copies ``piqmc/qmc.pyx``, ``piqmc/sa.pyx`` and ``piqmc/tools.pyx``
from the reference tree into ``oracle/_ref/piqmc_ref/`` (git-ignored build
output, never committed), applies the two one-line compatibility shims listed in
``SHIMS`` and cythonizes them with ``language_level=2`` into C.  The shims do not
change the arithmetic of any path:

* ``np.int_t`` -> ``np.int64_t``: NumPy 2 removed ``int_t`` from its ``.pxd``
  (reference ``piqmc/qmc.pyx:90``, ``:194``; ``piqmc/sa.pyx:91``); on LP64 the
  old ``int_t`` was ``long`` = int64, so the permutation buffer type is unchanged.
* ``J.iterkeys()`` -> ``J.keys()``: Python 3 dicts have no ``iterkeys``
  (reference ``piqmc/tools.pyx:84``).

``compile`` (needs gcc, Python and NumPy headers; runs on any host, including
one without Cython).  Compiles the generated C into extension modules with the
flags setuptools would use plus ``-fopenmp`` (reference ``setup.py:9-19``).

Usage::

    python oracle/build_ref.py            # generate (if the reference exists) + compile
    python oracle/build_ref.py compile    # compile previously generated C only
"""
import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("PIQMC_REFERENCE", "/root/reference")
OUT = os.path.join(HERE, "_ref")
PKG = os.path.join(OUT, "piqmc_ref")
MODULES = ("qmc", "sa", "tools")
SHIMS = (
    ("np.int_t", "np.int64_t"),
    ("J.iterkeys()", "J.keys()"),
)


def generate():
    """Copy the reference ``.pyx`` files into the build dir, apply ``SHIMS``, cythonize."""
    from Cython.Build import cythonize
    import numpy

    os.makedirs(PKG, exist_ok=True)
    with open(os.path.join(PKG, "__init__.py"), "w") as f:
        f.write("# compiled copy of the reference piqmc modules (parity checker only)\n")
    sources = []
    for mod in MODULES:
        src = os.path.join(REF_ROOT, "piqmc", mod + ".pyx")
        with open(src) as f:
            text = f.read()
        for old, new in SHIMS:
            text = text.replace(old, new)
        dst = os.path.join(PKG, mod + ".pyx")
        with open(dst, "w") as f:
            f.write(text)
        sources.append(dst)
    cwd = os.getcwd()
    os.chdir(OUT)
    try:
        cythonize([os.path.join("piqmc_ref", m + ".pyx") for m in MODULES],
                  compiler_directives={"language_level": 2},
                  include_path=[numpy.get_include()], quiet=True, force=True)
    finally:
        os.chdir(cwd)


def _compile_one(mod):
    import numpy

    csrc = os.path.join(PKG, mod + ".c")
    out = os.path.join(PKG, mod + sysconfig.get_config_var("EXT_SUFFIX"))
    flags = (sysconfig.get_config_var("CFLAGS") or "-O2").split()
    cmd = (["gcc"] + flags + ["-fPIC", "-shared", "-fopenmp", "-w",
            "-DNPY_NO_DEPRECATED_API=NPY_1_7_API_VERSION",
            "-I", sysconfig.get_paths()["include"], "-I", numpy.get_include(),
            csrc, "-o", out, "-lm"])
    subprocess.check_call(cmd)
    return out


def compile_ref():
    """Compile the generated C (no Cython needed)."""
    missing = [m for m in MODULES if not os.path.exists(os.path.join(PKG, m + ".c"))]
    if missing:
        raise FileNotFoundError("generated reference C missing for %s; run the generate stage "
                                "where the reference tree is mounted" % ", ".join(missing))
    with ThreadPoolExecutor(len(MODULES)) as ex:
        return list(ex.map(_compile_one, MODULES))


def available():
    """True when the compiled reference modules import in this interpreter."""
    return all(os.path.exists(os.path.join(PKG, m + sysconfig.get_config_var("EXT_SUFFIX")))
               for m in MODULES)


def main(argv):
    stage = argv[1] if len(argv) > 1 else "all"
    if stage in ("all", "generate") and os.path.isdir(os.path.join(REF_ROOT, "piqmc")):
        generate()
    if stage in ("all", "compile"):
        compile_ref()


if __name__ == "__main__":
    main(sys.argv)
