"""The ctypes mirrors of the C structs (dxtb_gb300/_lib.py) have the layout
the C compiler gives the structs of include/gbxtb.h: size and the offset of
every field, from a small C program built with the host compiler.  No
device is needed."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import pytest

from dxtb_gb300 import _lib

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.parametrize("cname, mirror", [("gbxtb_options", _lib.Options), ("gbxtb_params", _lib.Params)])
def test_struct_layout_matches_header(tmp_path, cname, mirror):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = [f[0] for f in mirror._fields_]
    lines = [f'  printf("{f} %zu\\n", offsetof({cname}, {f}));' for f in fields]
    src = tmp_path / "layout.c"
    src.write_text("#include <stdio.h>\n#include <stddef.h>\n#include \"gbxtb.h\"\nint main(void) {\n"
                   f'  printf("__size__ %zu\\n", sizeof({cname}));\n' + "\n".join(lines) + "\n  return 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True, capture_output=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                       text=True).stdout.splitlines())
    assert int(out["__size__"]) == C.sizeof(mirror)
    for f in fields:
        assert int(out[f]) == getattr(mirror, f).offset, f


def test_torch_op_option_vectors_match_the_unpacking():
    """calculator._pack_options writes the option fields in the order
    csrc/torch_ops.cpp reads them back (o.<field> = io[i] / fo[i])."""
    import re

    from dxtb_gb300.calculator import _pack_options, engine_options, resolve_opts

    text = (ROOT / "dxtb_gb300" / "csrc" / "torch_ops.cpp").read_text()
    iorder = {int(i): f for f, i in re.findall(r"o\.(\w+) = \(int32_t\)io\[(\d+)\]", text)}
    forder = {int(i): f for f, i in re.findall(r"o\.(\w+) = fo\[(\d+)\]", text)}
    opt = engine_options(resolve_opts({"exclude": ["disp"]}), forces=True)
    # give every field a distinct value, then check each lands at its index
    for k, (name, typ) in enumerate(_lib.Options._fields_):
        setattr(opt, name, (k + 1) if typ is C.c_int32 else (k + 1) * 0.5)
    iopts, fopts = _pack_options(opt)
    assert len(iopts) == len(iorder) and len(fopts) == len(forder)
    for i, f in iorder.items():
        assert iopts[i] == getattr(opt, f), (i, f)
    for i, f in forder.items():
        assert fopts[i] == getattr(opt, f), (i, f)
