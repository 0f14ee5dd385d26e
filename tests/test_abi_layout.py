"""Every struct of include/lqt.h that the Python side mirrors with ctypes has
the same size and the same field offsets in both: a C program compiled
against the header (as C, with gcc) prints them."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def mirrors():
    from lqt1_gb300 import _native as N
    from lqt1_gb300 import geometry as G
    from lqt1_gb300 import surrogate as S
    return {"lqt_model": N.Model, "lqt_instance": N.Instance, "lqt_batch_params": N.BatchParams,
            "lqt_geometry": N.Geometry, "lqt_protocol": N.Protocol, "lqt_sim_params": N.SimParams,
            "lqt_sur_config": N.SurConfig, "lqt_ventricle_spec": G.VentricleSpec,
            "lqt_geom_file_spec": G.GeomFileSpec, "lqt_sur_ranges": S.SurRanges}


def test_struct_layouts_match_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    ms = mirrors()
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "lqt.h"', "int main(void) {"]
    for cname, cls in ms.items():
        offs = " ".join(f"%zu" for _ in cls._fields_)
        args = ", ".join(f"offsetof({cname}, {f[0]})" for f in cls._fields_)
        lines.append(f'    printf("{cname} %zu {offs}\\n", sizeof({cname}), {args});')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    got = {}
    for ln in out.splitlines():
        name, *nums = ln.split()
        got[name] = [int(x) for x in nums]
    import ctypes as C
    for cname, cls in ms.items():
        want = [C.sizeof(cls)] + [getattr(cls, f[0]).offset for f in cls._fields_]
        assert got[cname] == want, (cname, got[cname], want)
