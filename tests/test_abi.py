"""The C ABI library: it loads without a GPU and exports every symbol the header declares."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT


def header_symbols():
    text = open(os.path.join(ROOT, "include", "salty_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(salty_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_python_binding_set(salty_lib):
    import salty_gb300
    assert header_symbols() == sorted(salty_gb300.EXPORTS)


def test_library_exports_every_declared_symbol(salty_lib):
    import salty_gb300
    out = subprocess.run(["nm", "-D", "--defined-only", salty_gb300.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (salty_[a-z0-9_]+)", out))
    missing = [s for s in header_symbols() if s not in exported]
    assert not missing, missing
    for s in header_symbols():
        assert hasattr(salty_lib, s)


def test_abi_version(salty_lib):
    assert salty_lib.salty_abi_version() == 2


def test_context_without_gpu_fails_cleanly(salty_lib):
    import torch
    import salty_gb300
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(salty_gb300.SaltyError) as e:
        salty_gb300.Context(0)
    assert e.value.status == salty_gb300.ERR_CUDA


def test_generators_validate_arguments(salty_lib):
    import ctypes as C
    assert salty_lib.salty_microbench_soup(1, -1, None) == 1
    assert salty_lib.salty_microbench_rays(1, 5, C.c_float(1e-4), None) == 1
    assert salty_lib.salty_microbench_soup(1, 0, None) == 0


def test_null_context_is_rejected(salty_lib):
    assert salty_lib.salty_bvh_build(None, None, None, None) == 1
    assert salty_lib.salty_trace(None, None, None, 0, 0, None) == 1
    assert salty_lib.salty_render(None, None, None, None, None, None, None) == 1
    assert salty_lib.salty_last_error(None) == b"null context"


def test_microbench_rays_are_unit_and_aimed_at_the_cube(salty_lib):
    import salty_gb300
    r = salty_gb300.microbench_rays(3, 10000, 1e-4)
    o, d = r[:, 0:3], r[:, 4:7]
    np.testing.assert_allclose(np.linalg.norm(o - 0.5, axis=1), 2.0, rtol=1e-6)
    np.testing.assert_allclose(np.linalg.norm(d, axis=1), 1.0, rtol=1e-6)
    assert np.all(r[:, 3] == np.float32(1e-4)) and np.all(np.isinf(r[:, 7]))
    # origin on the sphere is uniform: mean near the centre
    assert np.all(np.abs(o.mean(axis=0) - 0.5) < 0.05)


def test_header_is_plain_c99_and_links(salty_lib, tmp_path):
    """A C host (an FFI binding, a C caller) includes salty_gpu.h as strict C99 and links the
    library; the version query needs no GPU."""
    import shutil
    import salty_gb300
    if not shutil.which("gcc"):
        pytest.skip("no C compiler")
    src = tmp_path / "abi.c"
    src.write_text('#include "salty_gpu.h"\n'
                   "int main(void) { salty_ctx* c = 0; (void)c; return salty_abi_version() > 0 ? 0 : 1; }\n")
    exe = str(tmp_path / "abi")
    libdir = os.path.dirname(salty_gb300.LIB_PATH)
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Wpedantic", "-Werror",
                        f"-I{os.path.join(ROOT, 'include')}", str(src), f"-L{libdir}", "-lsalty_gpu",
                        f"-Wl,-rpath,{libdir}", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert subprocess.run([exe]).returncode == 0


def test_python_structs_match_the_header_layout(salty_lib, tmp_path):
    """Every ctypes mirror of a header struct has the C struct's size and each field its
    offset, as a C compiler lays them out (a field added on one side only would make the
    library read past the caller's struct)."""
    import ctypes
    import shutil
    import salty_gb300 as S
    if not shutil.which("gcc"):
        pytest.skip("no C compiler")
    pairs = [("salty_material", S.Material), ("salty_camera", S.Camera), ("salty_scene_desc", S.SceneDesc),
             ("salty_texture", S.Texture), ("salty_instance", S.Instance), ("salty_sphere", S.Sphere),
             ("salty_build_opts", S.BuildOpts), ("salty_bvh_info", S.BvhInfo),
             ("salty_trace_stats", S.TraceStats), ("salty_render_opts", S.RenderOpts),
             ("salty_render_stats", S.RenderStats), ("salty_mesh", S.Mesh), ("salty_tuning", S.Tuning)]
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "salty_gpu.h"', "int main(void) {"]
    for cname, cls in pairs:
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'    printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = str(tmp_path / "layout")
    r = subprocess.run(["gcc", "-std=c99", f"-I{os.path.join(ROOT, 'include')}", str(src), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = {}
    for line in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.splitlines():
        name, field, value = line.split()
        got[(name, field)] = int(value)
    for cname, cls in pairs:
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)
