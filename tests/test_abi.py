"""The C-ABI library builds, loads and exports every symbol the headers
declare; host-side argument checks run without a GPU (CPU)."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            names |= set(re.findall(r"^\s*(?:const\s+char\s*\*|sf_status|uint32_t|void)\s+(sf_\w+)\s*\(", text, re.M))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from syfrack_gb300 import _lib, build

    build.build()
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    names = declared_symbols()
    assert len(names) >= 30
    path = os.path.join(ROOT, "syfrack_gb300", "libsyfrack_gpu.so")
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (sf_\w+)$", out, re.M))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(lib, n)


def test_python_binding_covers_the_abi():
    from syfrack_gb300._lib import SIGNATURES

    assert sorted(SIGNATURES) == declared_symbols()


def test_status_strings(lib):
    assert lib.sf_status_string(0) == b"SF_OK"
    assert lib.sf_status_string(9) == b"SF_ERR_CHECKPOINT"
    assert lib.sf_status_string(99) == b"SF_ERR_UNKNOWN"
    assert lib.sf_abi_version() >> 16 == 1


def test_film_planes_struct_matches_the_header(lib):
    """sf_film_planes at ABI 1.1: seven plane pointers, the colour plane last."""
    import ctypes as C
    from syfrack_gb300._lib import sf_film_planes

    assert lib.sf_abi_version() & 0xFFFF >= 1
    assert [f[0] for f in sf_film_planes._fields_] == ["accum", "depth", "aux", "volume", "moments", "surface",
                                                       "color"]
    assert C.sizeof(sf_film_planes) == 7 * C.sizeof(C.c_void_p)
    header = open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "include", "syfrack_gpu.h")).read()
    body = header[header.index("typedef struct sf_film_planes"):header.index("} sf_film_planes;")]
    assert body.count("float*") == 7


def test_null_arguments_are_rejected(lib):
    assert lib.sf_context_create(0, 0, None) == 1  # SF_ERR_INVALID
    assert lib.sf_graph_compile(None, None, None) == 1
    assert lib.sf_session_dispatch(None, __import__("syfrack_gb300").abi.sf_tile(0, 0, 1, 1, 0), 1) == 1
    assert lib.sf_last_error() != b""


def test_render_config_struct_matches_the_header(lib):
    """sf_render_config at ABI 1.2: the hit epsilon follows samples_per_dispatch."""
    from syfrack_gb300 import abi

    assert lib.sf_abi_version() == (1 << 16) | 6
    assert [f[0] for f in abi.sf_render_config._fields_][-1] == "hit_epsilon"
    assert C.sizeof(abi.sf_render_config) == 10 * 4
    header = open(os.path.join(ROOT, "include", "syfrack_gpu.h")).read()
    body = header[header.index("typedef struct sf_render_config"):header.index("} sf_render_config;")]
    assert body.rstrip().endswith("float hit_epsilon;")


def test_deep_zoom_frames_beyond_2_31_pixels_are_refused(lib):
    """The perturbation kernel counts pixels in 32 bits: the allocation-free entry
    point refuses larger frames before it touches the device (no GPU needed)."""
    from syfrack_gb300._lib import sf_deep_zoom_desc

    d = sf_deep_zoom_desc()
    d.width, d.height, d.max_iter, d.bailout, d.width_units = 65536, 32769, 100, 2.0, 1e-3
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    assert lib.sf_deep_zoom_noalloc(C.byref(d), dummy, dummy, None) == 1  # SF_ERR_INVALID
    assert b"2^31" in lib.sf_last_error()


def test_scene_descriptor_layout_matches_the_header(tmp_path):
    """ABI 1.3 appends finish details, orbit colouring, optics and the texture to
    sf_scene_desc: the ctypes mirror has the C compiler's sizes and offsets."""
    import subprocess

    from syfrack_gb300 import abi

    src = tmp_path / "layout.c"
    src.write_text("""
#include <stdio.h>
#include <stddef.h>
#include "syfrack_gpu.h"
int main(void) {
    printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(sf_scene_desc), offsetof(sf_scene_desc, fog),
           offsetof(sf_scene_desc, details), offsetof(sf_scene_desc, dune_wind),
           offsetof(sf_scene_desc, coloring_orbit), offsetof(sf_scene_desc, optics),
           offsetof(sf_scene_desc, texture), sizeof(sf_texture), offsetof(sf_texture, ramp), sizeof(sf_optics));
    return 0;
}
""")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    S = abi.sf_scene_desc
    want = [C.sizeof(S), S.fog.offset, S.details.offset, S.dune_wind.offset, S.coloring_orbit.offset,
            S.optics.offset, S.texture.offset, C.sizeof(abi.sf_texture), abi.sf_texture.ramp.offset,
            C.sizeof(abi.sf_optics)]
    assert got == want
