"""Test infrastructure only (oracle): a host-memory stand-in for the ``pyopencl`` package.

The reference (SeaRay) drives its UPPE path through PyOpenCL.  Neither PyOpenCL nor an OpenCL
runtime exists in this container, so this package supplies the small part of the PyOpenCL API the
reference's UPPE modules call (``modules/init.py:5-62``, ``modules/uppe_kernel.py``,
``modules/grid_tools.py:198-358``, ``modules/ionization.py:26-34,131-150``):

* ``Program(ctx, text).build()`` compiles the OpenCL C text it is given as C++ with g++ and
  OpenMP (``clshim.h`` supplies ``double2`` and the work-item functions), and exposes every
  ``__kernel`` as ``prog.Name(queue, global_size, local_size, *args)``;
* ``pyopencl.array`` holds device arrays as NumPy arrays in host memory.

It lets the reference's own unmodified Python and its own kernels run on host cores, in FP64, to
produce golden vectors.  It is never imported by the product package.
"""
import ctypes
import hashlib
import os
import pathlib
import re
import subprocess

import numpy as np

VERSION = (2024, 1, 0)
VERSION_TEXT = "refshim"

_HERE = pathlib.Path(__file__).resolve().parent
_SHIM_DIR = _HERE.parent
_OUT_DIR = _SHIM_DIR.parent / "_ref"


class device_type:
    ALL = 0xFFFFFFFF
    CPU = 2
    GPU = 4


class Device:
    name = "host cores (refshim)"
    double_fp_config = 1
    extensions = "cl_khr_fp64"

    def get_info(self, *a, **k):
        return None


class Platform:
    name = "refshim"

    def get_devices(self, *a, **k):
        return [Device()]


def get_platforms():
    return [Platform()]


class Context:
    def __init__(self, devices=None, *a, **k):
        self.devices = devices or [Device()]


class CommandQueue:
    def __init__(self, ctx=None, *a, **k):
        self.context = ctx

    def finish(self):
        return None

    def flush(self):
        return None


class _KernelSig:
    __slots__ = ("name", "kinds")

    def __init__(self, name, kinds):
        self.name = name
        self.kinds = kinds


_KERNEL_RE = re.compile(r"__kernel\s+void\s+(\w+)\s*\(([^)]*)\)", re.S)


def _strip_comments(text):
    # parameter lists may carry comments, some with parentheses (rotations.cl:88-98)
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


def _parse_kernels(text):
    sigs = []
    for m in _KERNEL_RE.finditer(_strip_comments(text)):
        name = m.group(1)
        params = [p.strip() for p in m.group(2).split(",") if p.strip()]
        decls = []
        kinds = []
        for p in params:
            pname = re.findall(r"(\w+)\s*$", p)[0]
            ctype = p[: p.rfind(pname)].strip()
            decls.append((ctype, pname))
            if "*" in ctype:
                kinds.append("ptr")
            elif "Int" in ctype or re.search(r"\bint\b", ctype):
                kinds.append("int")
            else:
                kinds.append("double")
        sigs.append((name, decls, kinds))
    return sigs


def _launcher_source(sigs):
    out = ["\n// ---- launchers generated by the refshim ----\n"]
    for name, decls, _ in sigs:
        out.append(f'extern "C" void clshim_launch_{name}(int dims, const long* gs, void** argv) {{\n')
        for i, (ctype, _) in enumerate(decls):
            out.append(f"  {ctype} a{i} = *({ctype}*)argv[{i}];\n")
        out.append("  const long n0 = gs[0], n1 = dims > 1 ? gs[1] : 1, n2 = dims > 2 ? gs[2] : 1;\n")
        out.append("  #pragma omp parallel for collapse(3) schedule(static)\n")
        out.append("  for (long i = 0; i < n0; i++) for (long j = 0; j < n1; j++) for (long k = 0; k < n2; k++) {\n")
        out.append("    clshim_gsize[0] = n0; clshim_gsize[1] = n1; clshim_gsize[2] = n2;\n")
        out.append("    clshim_gid[0] = i; clshim_gid[1] = j; clshim_gid[2] = k;\n")
        args = ", ".join(f"a{i}" for i in range(len(decls)))
        out.append(f"    {name}({args});\n  }}\n}}\n")
    return "".join(out)


def _translate(text):
    # OpenCL C vector literals "(double2)(x,y)" are constructor calls in C++.
    return re.sub(r"\(\s*tw_Complex\s*\)\s*\(", "tw_Complex(", text)


class _Kernel:
    def __init__(self, lib, name, kinds):
        self.fn = getattr(lib, f"clshim_launch_{name}")
        self.fn.restype = None
        self.fn.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_void_p)]
        self.name = name
        self.kinds = kinds

    def __call__(self, queue, global_size, local_size, *args):
        if len(args) != len(self.kinds):
            raise TypeError(f"{self.name}: expected {len(self.kinds)} args, got {len(args)}")
        gs = tuple(int(g) for g in global_size)
        keep = []
        argv = (ctypes.c_void_p * len(args))()
        for i, (a, kind) in enumerate(zip(args, self.kinds)):
            if kind == "ptr":
                arr = a.base_array if hasattr(a, "base_array") else a
                if not arr.flags["C_CONTIGUOUS"]:
                    raise ValueError(f"{self.name}: argument {i} is not contiguous")
                v = ctypes.c_void_p(arr.ctypes.data)
            elif kind == "int":
                v = ctypes.c_int(int(a))
            else:
                v = ctypes.c_double(float(a))
            keep.append(v)
            argv[i] = ctypes.cast(ctypes.pointer(v), ctypes.c_void_p)
        gsa = (ctypes.c_long * 3)(*(gs + (1,) * (3 - len(gs))))
        self.fn(len(gs), gsa, argv)


class Program:
    def __init__(self, ctx, text):
        self.ctx = ctx
        self.text = text
        self._kernels = {}

    def build(self, *a, **k):
        sigs = _parse_kernels(self.text)
        src = '#include "clshim.h"\n' + _translate(self.text) + _launcher_source(sigs)
        digest = hashlib.sha1(src.encode()).hexdigest()[:16]
        _OUT_DIR.mkdir(parents=True, exist_ok=True)
        so = _OUT_DIR / f"cl_{digest}.so"
        if not so.exists():
            cpp = _OUT_DIR / f"cl_{digest}.cpp"
            cpp.write_text(src)
            tmp = _OUT_DIR / f"cl_{digest}.{os.getpid()}.so"
            cmd = ["g++", "-O2", "-fopenmp", "-shared", "-fPIC", "-Wno-unknown-pragmas",
                   "-I", str(_SHIM_DIR), "-o", str(tmp), str(cpp)]
            subprocess.run(cmd, check=True)
            os.replace(tmp, so)
        lib = ctypes.CDLL(str(so))
        for name, _, kinds in sigs:
            self._kernels[name] = _Kernel(lib, name, kinds)
        return self

    def __getattr__(self, name):
        ks = self.__dict__.get("_kernels", {})
        if name in ks:
            return ks[name]
        raise AttributeError(name)


from . import array  # noqa: E402,F401
