"""The C ABI driven from C (tests/c/render_file.c, built with gcc against include/rast.h and
librast.so): the frame equals the oracle's bit for bit."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from rusterizer_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _write_scene(path, s):
    d = s["draws"][0]
    tex = np.ascontiguousarray(s["textures"][0], np.uint8)
    with open(path, "wb") as f:
        f.write(np.array([s["width"], s["height"], s["msaa"], len(d["pos"]), len(d["idx"]),
                          tex.shape[1], tex.shape[0], d.get("fs", 0)], np.int32).tobytes())
        f.write(np.array([s["clear_depth"]], np.float32).tobytes())
        for m in (d["world"], s["view"], s["proj"]):
            f.write(np.ascontiguousarray(m, np.float32).tobytes())
        f.write(np.ascontiguousarray(d["pos"], np.float32).tobytes())
        f.write(np.ascontiguousarray(d["uv"], np.float32).tobytes())
        f.write(np.ascontiguousarray(d["idx"], np.uint32).tobytes())
        f.write(tex.tobytes())


@pytest.mark.parametrize("make", [scenes.config0, lambda: scenes.small_soup(5)])
def test_c_program_renders_like_the_oracle(tmp_path, make):
    s = make()
    exe = tmp_path / "render_file"
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run(["gcc", "-O2", "-std=c11", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "c", "render_file.c"), "-o", str(exe), "-L", libdir, "-lrast",
                    "-Wl,-rpath," + libdir], check=True)
    _write_scene(tmp_path / "scene.bin", s)
    subprocess.run([str(exe), str(tmp_path / "scene.bin"), str(tmp_path / "out.bin")], check=True)
    raw = np.fromfile(tmp_path / "out.bin", np.uint32)
    img, status = raw[:-1].reshape(s["height"], s["width"]), int(raw[-1])
    assert status in (_lib.OK, _lib.TEXTURE_OOB)
    ref, *_ = oracle.render_scene(s)
    assert (img == ref).all()
