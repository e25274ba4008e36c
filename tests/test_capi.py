"""C ABI surface (CPU): the library loads, exports every declared symbol, and
the Python mirrors of the header agree with it."""
from __future__ import annotations

import ctypes as C
import re
import subprocess
import textwrap
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "covof_gpu.h"


def _declared():
    txt = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+(covof_\w+)\s*\(", txt, re.M)))


@pytest.fixture(scope="module")
def lib(pkg):
    import __graft_entry__ as ge
    ge._load_build_module().build()
    return pkg.capi.load_library()


def test_library_exports_every_declared_symbol(lib):
    declared = _declared()
    assert len(declared) >= 30
    for name in declared:
        assert hasattr(lib, name), name


def test_python_mirror_covers_the_header(pkg):
    assert sorted(pkg.capi.exported_symbols()) == _declared()


@pytest.mark.parametrize("cname,pyname", [("covof_params", "Params"), ("covof_run_stats", "RunStats")])
def test_struct_layout_matches_c(pkg, tmp_path, cname, pyname):
    struct = getattr(pkg.capi, pyname)
    src = tmp_path / "probe.c"
    fields = [f for f, _ in struct._fields_]
    body = "\n".join(f'  printf("%s %zu\\n", "{f}", offsetof({cname}, {f}));' for f in fields)
    src.write_text(textwrap.dedent(f"""
        #include <stdio.h>
        #include <stddef.h>
        #include "{HEADER}"
        int main(void) {{
          printf("sizeof %zu\\n", sizeof({cname}));
        {body}
          return 0;
        }}"""))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-o", str(exe), str(src)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                         check=True).stdout.splitlines())
    assert int(out["sizeof"]) == C.sizeof(struct)
    for f in fields:
        assert int(out[f]) == getattr(struct, f).offset, f


def test_field_ids_match_c(pkg, tmp_path):
    src = tmp_path / "ids.c"
    names = [f"COVOF_FIELD_{n.upper()}" for n in pkg.capi.FIELD_NAMES]
    body = "\n".join(f'  printf("%d\\n", {n});' for n in names)
    src.write_text(f'#include <stdio.h>\n#include "{HEADER}"\nint main(void) {{\n{body}\n'
                   f'  printf("%d\\n", COVOF_NFIELDS);\n  return 0;\n}}\n')
    exe = tmp_path / "ids"
    subprocess.run(["gcc", "-o", str(exe), str(src)], check=True)
    vals = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                           check=True).stdout.split()]
    assert vals == list(range(len(names))) + [len(names)]


def test_default_params_match_python_twin(lib, pkg):
    a = pkg.capi.default_params(40, 30, 2.0, 1.5)
    b = pkg.cases.make_params(40, 30, 2.0, 1.5)
    assert a.as_dict() == b.as_dict()


def test_strerror_names_every_status(lib, pkg):
    for s in range(9):
        assert lib.covof_strerror(s)
    assert lib.covof_abi_version() == 1
