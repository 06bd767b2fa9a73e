"""Build the reference's own compiled kernels for timing and checking: holodeck's two Cython modules.

TEST INFRASTRUCTURE ONLY (the reference arm of ``bench.py`` and the CPU baseline).  Nothing in the
``holodeck_gb300`` product imports, links or runs what this recipe builds.

The reference's compiled path is ``holodeck/cyutils.pyx`` (the Poisson realizations with the
loudest-source split, cyutils.pyx:1220-1344) and ``holodeck/sams/sam_cyutils.pyx`` (hardening
normalisation, differential number, integration, sam_cyutils.pyx:115-899), built by the reference's
``setup.py:32-70`` against numpy's ``npyrandom`` / ``npymath``.  Two steps, because the machine
that holds the reference sources and Cython is not the one that runs the timing:

1. ``generate`` (needs ``HOLODECK_REF_SRC``, the holodeck source root, and Cython): translates the
   two ``.pyx`` files, read where they lie, to C with the reference's compiler directives
   (``language_level=3``) and module names ``holodeck.cyutils`` / ``holodeck.sams.sam_cyutils``.
   The one change is the Cython-3 token ``long(normal_threshold)`` -> ``int(normal_threshold)``
   (holodeck/cyutils.pyx:855; Cython 3 has no ``long`` builtin), applied to a temporary copy.
   Output: ``oracle/_ref/gen/*.c`` (generated code, not committed).
2. ``compile`` (any machine with gcc, Python headers and numpy): compiles those C files into
   importable extension modules under ``oracle/_ref/pkg/holodeck/`` (links ``npyrandom`` and
   ``npymath`` as setup.py does) and writes the package's import stand-in (:mod:`oracle.ref_stub`),
   which gives ``sam_cyutils`` the only names it looks up in its package at run time
   (``holodeck.hardening.Fixed_Time_2PL_SAM`` / ``Hard_GW`` for its isinstance dispatch).

``load()`` imports the compiled modules from ``oracle/_ref/pkg``.
"""

import concurrent.futures
import os
import shutil
import subprocess
import sys
import sysconfig
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
GEN_DIR = os.path.join(REF_DIR, "gen")
PKG_DIR = os.path.join(REF_DIR, "pkg")
MODULES = {   # module name -> (path of the .pyx inside the holodeck source root, generated C file)
    "holodeck.cyutils": (os.path.join("holodeck", "cyutils.pyx"), "cyutils.c"),
    "holodeck.sams.sam_cyutils": (os.path.join("holodeck", "sams", "sam_cyutils.pyx"), "sam_cyutils.c"),
}


def generated():
    return all(os.path.exists(os.path.join(GEN_DIR, c)) for _, c in MODULES.values())


def generate(src_root=None):
    """Translate the reference's .pyx files to C into oracle/_ref/gen (step 1)."""
    src_root = src_root or os.environ.get("HOLODECK_REF_SRC")
    if not src_root:
        raise RuntimeError("set HOLODECK_REF_SRC to the holodeck source root")
    os.makedirs(GEN_DIR, exist_ok=True)
    with tempfile.TemporaryDirectory() as tmp:
        # the include tree Cython resolves `cimport holodeck.cyutils` against
        os.makedirs(os.path.join(tmp, "holodeck", "sams"))
        for rel in ["cyutils.pxd", "cyutils.pyx", os.path.join("sams", "sam_cyutils.pyx")]:
            shutil.copy(os.path.join(src_root, "holodeck", rel), os.path.join(tmp, "holodeck", rel))
        for d in ["holodeck", os.path.join("holodeck", "sams")]:
            open(os.path.join(tmp, d, "__init__.py"), "w").close()
        pyx = os.path.join(tmp, "holodeck", "cyutils.pyx")
        os.chmod(pyx, 0o644)
        text = open(pyx).read()
        assert text.count("long(normal_threshold)") == 1
        with open(pyx, "w") as fh:
            fh.write(text.replace("long(normal_threshold)", "int(normal_threshold)"))
        for mod, (rel, cfile) in MODULES.items():
            subprocess.run([sys.executable, "-m", "cython", "-3", "--module-name", mod, "-I", tmp,
                            os.path.join(tmp, rel), "-o", os.path.join(GEN_DIR, cfile)], check=True,
                           stdout=subprocess.DEVNULL)
    return GEN_DIR


def _ext_path(mod):
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    return os.path.join(PKG_DIR, *mod.split(".")) + suffix


def compiled():
    return all(os.path.exists(_ext_path(m)) for m in MODULES)


def compile(force=False):
    """Compile the generated C into extension modules under oracle/_ref/pkg (step 2)."""
    if not generated():
        raise RuntimeError("oracle/_ref/gen holds no generated C: run `python oracle/ref_build.py generate` "
                           "where the reference sources and Cython are")
    import numpy as np
    from oracle import ref_stub
    os.makedirs(os.path.join(PKG_DIR, "holodeck", "sams"), exist_ok=True)
    with open(os.path.join(PKG_DIR, "holodeck", "__init__.py"), "w") as fh:
        fh.write(ref_stub.PACKAGE_INIT)
    open(os.path.join(PKG_DIR, "holodeck", "sams", "__init__.py"), "w").close()
    npinc = np.get_include()
    libdirs = [os.path.abspath(os.path.join(npinc, "..", "..", "random", "lib")),
               os.path.abspath(os.path.join(npinc, "..", "lib"))]
    pyinc = sysconfig.get_paths()["include"]

    def one(item):
        mod, (_, cfile) = item
        out = _ext_path(mod)
        src = os.path.join(GEN_DIR, cfile)
        if not force and os.path.exists(out) and os.path.getmtime(out) > os.path.getmtime(src):
            return out
        cmd = ["gcc", "-O2", "-shared", "-fPIC", "-fno-strict-aliasing", "-DNPY_NO_DEPRECATED_API=0",
               "-I", pyinc, "-I", npinc, src, "-o", out + ".tmp"]
        for d in libdirs:
            cmd += ["-L", d]
        cmd += ["-lnpyrandom", "-lnpymath", "-lm"]
        subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        os.replace(out + ".tmp", out)
        return out

    with concurrent.futures.ThreadPoolExecutor(2) as ex:
        return list(ex.map(one, MODULES.items()))


def load():
    """(cyutils, sam_cyutils) of the reference, compiled from its sources (compiles on first use)."""
    if not compiled():
        compile()
    if PKG_DIR not in sys.path:
        sys.path.insert(0, PKG_DIR)
    import holodeck.cyutils as cyutils
    import holodeck.sams.sam_cyutils as sam_cyutils
    return cyutils, sam_cyutils


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(HERE))
    step = sys.argv[1] if len(sys.argv) > 1 else "all"
    if step in ("generate", "all"):
        print(generate())
    if step in ("compile", "all"):
        print(compile(force=True))
