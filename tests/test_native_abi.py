"""The C-ABI library: it builds, loads, exports every entry point include/searay_uppe.h declares,
and the ctypes mirror of UppeConfig has the C layout.  No device calls (runs without a GPU)."""
import ctypes
import pathlib
import re
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "searay_uppe.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(uppe_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def built():
    from searay_gb300 import build
    build.build()
    from searay_gb300 import _native
    return _native.lib()


def test_exports_every_declared_symbol(built):
    from searay_gb300 import _native
    names = declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(built, n), n
    assert set(names) == set(_native.EXPORTS)


def test_config_struct_layout(tmp_path):
    from searay_gb300 import _native
    src = tmp_path / "probe.c"
    fields = [f[0] for f in _native.UppeConfig._fields_]
    body = "\n".join(f'printf("%zu ", offsetof(UppeConfig, {f}));' for f in fields)
    src.write_text(f'#include <stdio.h>\n#include <stddef.h>\n#include "searay_uppe.h"\n'
                   f'int main(void){{ {body} printf("%zu\\n", sizeof(UppeConfig)); return 0; }}\n')
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), "-o", str(exe), str(src)], check=True)
    out = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    offs = [getattr(_native.UppeConfig, f).offset for f in fields] + [ctypes.sizeof(_native.UppeConfig)]
    assert out == offs


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from searay_gb300 import _native
    monkeypatch.setattr(_native, "_LIB", None)
    monkeypatch.setattr(_native, "LIB_PATH", tmp_path / "absent.so")
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _native.lib()
