"""Build recipe for the compiled reference oracle (``oracle/_ref``).

This is test infrastructure.  It copies the reference PySPH snapshot
(``source/pysph`` of the reference tree, a Python 2 / Cython 0.14 code base)
into ``oracle/_ref/src``, applies mechanical Python 3 / Cython 3
compatibility edits (syntax and API renames only -- no change to any
arithmetic), and compiles the hot-path extension modules in place.  The
result is importable as ``pysph`` with ``oracle/_ref/src`` on ``sys.path``.

Nothing under ``oracle/_ref`` is committed.  The reference is used:

* to generate the golden fixtures under ``tests/golden`` (see
  ``tests/golden/make_golden.py``);
* to cross-check the C restatement in ``oracle/sph_oracle.c``;
* as the timed CPU baseline of ``bench.py --impl reference``.

Usage::

    python oracle/build_ref.py [--reference DIR] [--cythonize-only] [--jobs N]

``--cythonize-only`` stops after generating the C++ sources; ``--compile``
compiles previously generated sources without needing Cython or the
reference tree (used on a host that only has the generated files).
"""
import argparse
import os
import re
import shutil
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
SRC_OUT = os.path.join(REF_OUT, "src")

# Hot-path extension modules (module name -> .pyx path relative to src).
MODULES = [
    "pysph.base.carray", "pysph.base.point", "pysph.base.plane",
    "pysph.base.particle_array", "pysph.base.cell", "pysph.base.polygon_array",
    "pysph.base.nnps", "pysph.base.geometry", "pysph.base.kernels",
    "pysph.sph.sph_func", "pysph.sph.sph_calc", "pysph.sph.kernel_correction",
    "pysph.sph.funcs.basic_funcs", "pysph.sph.funcs.position_funcs",
    "pysph.sph.funcs.boundary_funcs", "pysph.sph.funcs.external_force",
    "pysph.sph.funcs.density_funcs", "pysph.sph.funcs.energy_funcs",
    "pysph.sph.funcs.viscosity_funcs", "pysph.sph.funcs.pressure_funcs",
    "pysph.sph.funcs.xsph_funcs", "pysph.sph.funcs.eos_funcs",
    "pysph.sph.funcs.adke_funcs", "pysph.sph.funcs.arithmetic_funcs",
    "pysph.solver.particle_generator",
]

# ---------------------------------------------------------------------------
# compatibility edits
# ---------------------------------------------------------------------------

def _fix_has_key(text):
    # a.has_key(k) -> (k in a)
    pat = re.compile(r"([A-Za-z_][\w\.]*(?:\[[^\[\]]*\])?)\.has_key\(([^()]*(?:\([^()]*\))?[^()]*)\)")
    return pat.sub(lambda m: "(%s in %s)" % (m.group(2), m.group(1)), text)


def _fix_common(text):
    text = _fix_has_key(text)
    text = text.replace(".iteritems()", ".items()")
    text = text.replace(".itervalues()", ".values()")
    text = text.replace(".iterkeys()", ".keys()")
    text = re.sub(r"\bxrange\(", "range(", text)
    # dict views used as lists
    text = re.sub(r"(self\.\w+)\.keys\(\) \+ (self\.\w+)\.keys\(\)",
                  r"list(\1.keys()) + list(\2.keys())", text)
    text = re.sub(r"self\.properties\.values\(\)\[0\]",
                  "list(self.properties.values())[0]", text)
    return text


def _fix_print(line):
    m = re.match(r"^(\s*)print\s+(?!\()(.*?)\s*$", line)
    if m and not m.group(2).startswith(("=", ",")):
        body = m.group(2)
        end = ""
        if body.endswith(","):
            body = body[:-1]
            end = ", end=' '"
        if body.startswith(">>"):
            return line
        return "%sprint(%s%s)\n" % (m.group(1), body, end)
    if re.match(r"^\s*print\s*$", line):
        return re.sub(r"print\s*$", "print()", line.rstrip("\n")) + "\n"
    return line


def _fix_py(text, local_modules):
    text = _fix_common(text)
    lines = []
    for line in text.splitlines(True):
        line = _fix_print(line)
        # raise E, msg  -> raise E(msg)
        m = re.match(r"^(\s*)raise\s+([\w\.]+)\s*,\s*(.+?)\s*$", line)
        if m:
            line = "%sraise %s(%s)\n" % (m.group(1), m.group(2), m.group(3))
        # except E, e: -> except E as e:
        line = re.sub(r"except\s+([\w\.\(\), ]+?)\s*,\s*(\w+)\s*:", r"except \1 as \2:", line)
        # implicit relative imports inside a package
        m = re.match(r"^(\s*)from\s+(\w+)((?:\.\w+)*)\s+import\s+(.*)$", line)
        if m and m.group(2) in local_modules:
            line = "%sfrom .%s%s import %s\n" % (m.group(1), m.group(2), m.group(3), m.group(4))
            m = None
        if m and False:
            line = "%sfrom .%s import %s\n" % (m.group(1), m.group(2), m.group(3))
        m = re.match(r"^(\s*)import\s+([\w ,]+?)\s*$", line)
        if m:
            names = [n.strip() for n in m.group(2).split(",")]
            if all(n in local_modules for n in names):
                line = "%sfrom . import %s\n" % (m.group(1), ", ".join(names))
        lines.append(line)
    text = "".join(lines)
    text = text.replace("import commands", "import subprocess as commands")
    text = re.sub(r"^import thread\b", "import _thread as thread", text, flags=re.M)
    text = re.sub(r"^import threading, thread$", "import threading, _thread as thread", text, flags=re.M)
    text = text.replace("sys.maxint", "sys.maxsize")
    text = re.sub(r"\bbasestring\b", "str", text)
    return text


PYX_EDITS = {
    # stdlib cimport moved to libc in Cython >= 0.15
    "base/carray.pyx": [("from stdlib cimport *", "from libc.stdlib cimport *")],
    "base/point.pyx": [
        ("cpdef inline double norm", "cpdef double norm"),
        ("DTYPE = numpy.float\n", "DTYPE = numpy.float64\n"),
        ("numpy.int_t", "numpy.int64_t"),
        ("dtype=numpy.int)", "dtype=numpy.int64)"),
        ("dtype=numpy.int]", "dtype=numpy.int64_t]"),
    ],
    "base/plane.pyx": [("DTYPE = numpy.float\n", "DTYPE = numpy.float64\n")],
    "base/kernels.pyx": [
        ("__gradient", "_kgradient"),
        ("dtype=numpy.float]", "dtype=numpy.float64_t]"),
    ],
    "base/kernels.pxd": [("__gradient", "_kgradient")],
    "base/particle_array.pyx": [
        ("cpdef int append_parray(self, ParticleArray parray):",
         "cpdef int append_parray(self, ParticleArray parray) except -1:"),
        ("cdef str prop_name, data_type\n        cdef object data, default\n",
         "cdef str prop_name = None, data_type = None\n        cdef object data = None, default = None\n"),
    ],
    "base/cell.pyx": [
        ("numpy.int_t", "numpy.int64_t"),
    ],
    "sph/funcs/external_force.pyx": [],
}


def _patch_particle_array(text):
    # PyString_AsString(data_type) comparisons -> plain string compares
    text = re.sub(r"strcmp\(PyString_AsString\((\w+)\),\s*'(\w+)'\)\s*==\s*0",
                  r"\1 == '\2'", text)
    text = re.sub(r"strcmp\(PyString_AsString\((\w+)\),\s*\"(\w+)\"\)\s*==\s*0",
                  r"\1 == '\2'", text)
    text = re.sub(r"for (\w+) in (self\.\w+|\w+)\.keys\(\)", r"for \1 in list(\2.keys())", text)
    text = re.sub(r"= (props|self\.properties)\.keys\(\)\s*$", r"= list(\1.keys())", text, flags=re.M)
    text = text.replace("%PyString_AsString(data_type)", "%data_type")
    text = re.sub(r"(\w+(?:\.\w+)*)\.values\(\)(?!\))", r"list(\1.values())", text)
    return text


def _patch_cell(text):
    text = text.replace("cpdef int update_status(self):", "cpdef int update_status(self) except -1:")
    text = re.sub(r"(cdef int get_potential_cells\(self, cPoint pnt, double radius,\s*list cell_list\))(:)",
                  r"\1 except -1\2", text)
    text = text.replace("self.cells_dict.values()", "list(self.cells_dict.values())")
    text = text.replace("PyDict_Values( self.cells_dict)", "list(self.cells_dict.values())")
    return text


def _patch_cell_pxd(text):
    text = re.sub(r"cpdef int update_status\(self\)(?! except)", "cpdef int update_status(self) except -1", text)
    text = re.sub(r"(cdef int get_potential_cells\(self, cPoint pnt, double radius,\s*list cell_list\))(?! except)",
                  r"\1 except -1", text)
    return text


def patch_tree(src_root):
    pkg = os.path.join(src_root, "pysph")
    for dirpath, _, files in os.walk(pkg):
        local = {os.path.splitext(f)[0] for f in files if f.endswith((".py", ".pyx"))}
        local |= {d for d in os.listdir(dirpath) if os.path.isfile(os.path.join(dirpath, d, "__init__.py"))}
        for f in files:
            path = os.path.join(dirpath, f)
            rel = os.path.relpath(path, pkg).replace(os.sep, "/")
            if f.endswith(".py"):
                with open(path) as fh:
                    text = fh.read()
                text = _fix_py(text, local)
                with open(path, "w") as fh:
                    fh.write(text)
            elif f.endswith((".pyx", ".pxd")):
                with open(path) as fh:
                    text = fh.read()
                if f.endswith(".pyx"):
                    text = _fix_common(text)
                for old, new in PYX_EDITS.get(rel, []):
                    text = text.replace(old, new)
                if rel == "base/particle_array.pyx":
                    text = _patch_particle_array(text)
                if rel == "base/cell.pyx":
                    text = _patch_cell(text)
                if rel == "base/cell.pxd":
                    text = _patch_cell_pxd(text)
                with open(path, "w") as fh:
                    fh.write(text)


# ---------------------------------------------------------------------------
# build
# ---------------------------------------------------------------------------

def copy_tree(reference):
    src = os.path.join(reference, "source", "pysph")
    if os.path.exists(SRC_OUT):
        shutil.rmtree(SRC_OUT)
    shutil.copytree(src, os.path.join(SRC_OUT, "pysph"),
                    ignore=shutil.ignore_patterns("*.png", "*.fig", "*.bak", "*.c", "*.cpp", "*.so"))


def cythonize_all(jobs):
    from Cython.Build import cythonize
    from setuptools import Extension
    import numpy
    exts = []
    for mod in MODULES:
        pyx = os.path.join(SRC_OUT, *mod.split(".")) + ".pyx"
        exts.append(Extension(mod, [pyx], include_dirs=[numpy.get_include()], language="c++"))
    cwd = os.getcwd()
    os.chdir(SRC_OUT)
    try:
        cythonize(exts, nthreads=jobs, include_path=[SRC_OUT, numpy.get_include()],
                  compiler_directives={"language_level": 2, "embedsignature": True,
                                       "legacy_implicit_noexcept": True,
                                       "cpow": True, "binding": False},
                  quiet=True)
    finally:
        os.chdir(cwd)


def _compile_one(mod):
    import numpy
    cpp = os.path.join(SRC_OUT, *mod.split(".")) + ".cpp"
    ext_suffix = sysconfig.get_config_var("EXT_SUFFIX")
    out = os.path.join(SRC_OUT, *mod.split(".")) + ext_suffix
    if os.path.exists(out) and os.path.getmtime(out) > os.path.getmtime(cpp):
        return mod, 0, ""
    cmd = ["g++", "-O2", "-fPIC", "-shared", "-w", "-ffp-contract=off",
           "-I" + sysconfig.get_paths()["include"], "-I" + numpy.get_include(),
           "-I" + SRC_OUT, cpp, "-o", out]
    p = subprocess.run(cmd, capture_output=True, text=True)
    return mod, p.returncode, p.stderr[-3000:]


def compile_all(jobs):
    failed = []
    with ThreadPoolExecutor(jobs) as ex:
        for mod, rc, err in ex.map(_compile_one, MODULES):
            if rc != 0:
                failed.append(mod)
                sys.stderr.write("FAILED %s\n%s\n" % (mod, err))
    if failed:
        raise SystemExit("reference build failed: %s" % failed)


STAMP = os.path.join(REF_OUT, "built.stamp")


def _up_to_date():
    if not os.path.exists(STAMP):
        return False
    with open(STAMP) as fh:
        recorded = fh.read().strip()
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    sos = [os.path.join(SRC_OUT, *m.split(".")) + ext for m in MODULES]
    return recorded == _recipe_id() and all(os.path.exists(x) for x in sos)


def _recipe_id():
    return "%s:%s" % (os.path.getmtime(os.path.abspath(__file__)), sysconfig.get_config_var("EXT_SUFFIX"))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--reference", default=os.environ.get("PYSPH_REFERENCE_TREE", "/root/reference"),
                    help="the reference's source tree (default: environment PYSPH_REFERENCE_TREE)")
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 4)
    ap.add_argument("--cythonize-only", action="store_true")
    ap.add_argument("--compile", action="store_true",
                    help="compile already generated C++ sources only")
    args = ap.parse_args()
    if not args.force and _up_to_date():
        print("reference oracle up to date in", SRC_OUT)
        return
    if not args.compile:
        if not os.path.isdir(args.reference):
            raise SystemExit("reference tree not found: %s" % args.reference)
        copy_tree(args.reference)
        patch_tree(SRC_OUT)
        cythonize_all(args.jobs)
        if args.cythonize_only:
            return
    compile_all(args.jobs)
    with open(STAMP, "w") as fh:
        fh.write(_recipe_id())
    print("reference oracle built in", SRC_OUT)


if __name__ == "__main__":
    main()
