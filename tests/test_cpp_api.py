"""The C++ host API (include/salty/pt.hpp): compiles against the C ABI everywhere, and on a
GPU renders through PathTracer::Run like a Salty host would."""
import os
import shutil
import struct
import subprocess
import zlib

import numpy as np
import pytest

from conftest import ROOT


def _compile(salty_lib, tmp_path, name="cornell_pt"):
    import salty_gb300
    if not shutil.which("g++"):
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / name)
    libdir = os.path.dirname(salty_gb300.LIB_PATH)
    r = subprocess.run(["g++", "-std=c++17", "-O2", f"-I{os.path.join(ROOT, 'include')}",
                        os.path.join(ROOT, "tests", "cpp", f"{name}.cpp"), f"-L{libdir}", "-lsalty_gpu",
                        f"-Wl,-rpath,{libdir}", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("name", ["cornell_pt", "textured_pt"])
def test_cpp_api_compiles_and_links(salty_lib, tmp_path, name):
    _compile(salty_lib, tmp_path, name)


def _read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        ln, = struct.unpack(">I", data[pos:pos + 4])
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + ln]
        crc, = struct.unpack(">I", data[pos + 8 + ln:pos + 12 + ln])
        assert zlib.crc32(typ + body) & 0xffffffff == crc
        if typ == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif typ == b"IDAT":
            idat += body
        pos += 12 + ln
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 3 * w)
    assert np.all(raw[:, 0] == 0)
    return raw[:, 1:].reshape(h, w, 3)


@pytest.mark.gpu
def test_cpp_pathtracer_run_renders_the_cornell_box(salty_lib, tmp_path, oracle):
    from oracle.oracle import PROFILE_PHYSICAL, SceneData
    from salty_gb300 import scenes
    exe = _compile(salty_lib, tmp_path)
    png = str(tmp_path / "final.png")
    r = subprocess.run([exe, png, "16"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    words = r.stdout.split()
    assert words[0] == "passes" and int(words[1]) == 16 and words[2] == "spp" and int(words[3]) == 64
    mean = np.array([float(x) for x in words[5:8]])
    img = _read_png(png)
    assert img.shape == (128, 128, 3) and img.max() <= 247 and img.mean() > 20
    # same scene, oracle estimator: image means agree to a few percent (64 spp each)
    c = scenes.cornell("baseline")
    # the C++ example has no boxes: drop them (the first 10 triangles are the walls)
    sd = SceneData(c["tri_pos"][:10], c["tri_nrm"][:10], c["tri_mat"][:10], c["materials"], c["light"], None,
                   c["sky"], c["camera"])
    tot, _ = oracle.render(sd, 64, 64, 64, 8, profile=PROFILE_PHYSICAL, seed=2)
    om = (tot / 64).reshape(-1, 3).mean(axis=0)
    np.testing.assert_allclose(mean, om, rtol=0.05)


@pytest.mark.gpu
def test_cpp_pathtracer_time_budget_grows_passes(salty_lib, tmp_path):
    """PathTracer::Run with a time budget and no pass limit (Salty's MaxRenderingSec loop):
    passes double while they fit, so the 0.5 s budget holds many more samples than passes
    of the first size would, and the image is a converged Cornell box."""
    exe = _compile(salty_lib, tmp_path)
    png = str(tmp_path / "budget.png")
    r = subprocess.run([exe, png, "0", "0.5"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    words = r.stdout.split()
    passes, spp = int(words[1]), int(words[3])
    # spp = 4 * (2^k - 1) + the repeats of the last size: far more than 4 per pass
    assert spp >= 16 * passes and spp % 4 == 0, (passes, spp)
    mean = np.array([float(x) for x in words[5:8]])
    assert np.all(np.isfinite(mean)) and mean.min() > 0
    assert _read_png(png).mean() > 20


@pytest.mark.gpu
def test_cpp_textures_environment_and_smd_instances(salty_lib, tmp_path):
    """AddTexture / SetColorMap / SetEnvironment / AddSmd (with and without a transform)
    from C++: the program renders and writes its PNG."""
    from salty_gb300 import scenes
    from test_smd import write_smd
    unit = scenes._icosphere(2).astype(np.float32).reshape(-1, 9)
    n = unit.shape[0]
    mesh = str(tmp_path / "ball.smd")
    write_smd(mesh, unit * 0.4 + np.tile([0, 0.4, 0], 3).astype(np.float32), unit, np.zeros((n, 6), np.float32),
              np.zeros(n, np.int32),
              [(4, {"diffuse": (0.7, 0.3, 0.2), "specular": (0.5, 0.5, 0.5), "power": 50.0, "emission": (0, 0, 0)})])
    exe = _compile(salty_lib, tmp_path, "textured_pt")
    png = str(tmp_path / "t.png")
    r = subprocess.run([exe, mesh, png, "4"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    words = r.stdout.split()
    assert words[0] == "passes" and int(words[1]) == 4
    mean = np.array([float(x) for x in words[3:6]])
    assert np.all(np.isfinite(mean)) and mean.min() > 0
    img = _read_png(png)
    assert img.shape == (64, 96, 3) and img.std() > 5  # textured floor, spheres, sky: not flat
