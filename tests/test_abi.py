"""The C ABI without a GPU: the library builds and loads, exports every entry point that
include/gartus_gpu.h declares, and the ctypes mirror has the header's struct layouts."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

from gartus_gb300 import abi
from gartus_gb300 import build as gbuild
from gartus_gb300._lib import EXPORTED_SYMBOLS, GartusError, lib

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "gartus_gpu.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\**\s+\**(gt_[a-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_builds_and_loads():
    path = gbuild.build()
    assert path.exists()
    assert lib().gt_abi_version() == abi.GT_ABI_VERSION


def test_every_declared_symbol_is_exported():
    declared = declared_functions()
    assert len(declared) >= 15
    assert sorted(EXPORTED_SYMBOLS) == declared
    out = subprocess.run(["nm", "-D", "--defined-only", str(gbuild.LIB)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\sT\s(gt_[a-z_0-9]+)$", out, flags=re.M))
    missing = [n for n in declared if n not in exported]
    assert not missing, missing


def test_struct_layouts_match_header(tmp_path):
    fields = {s.__name__: [f[0] for f in s._fields_] for s in abi.STRUCTS}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for name, fs in fields.items():
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for f in fs:
            lines.append(f'printf("{name}.{f} %zu\\n", offsetof({name}, {f}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", str(src), "-o", str(exe)], check=True)
    got = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                               check=True).stdout.splitlines())
    for s in abi.STRUCTS:
        assert int(got[s.__name__]) == C.sizeof(s), s.__name__
        for f in s._fields_:
            assert int(got[f"{s.__name__}.{f[0]}"]) == getattr(s, f[0]).offset, (s.__name__, f[0])


def test_constants_match_header(tmp_path):
    # every GT_* integer constant of the Python mirror has the header's value
    names = [n for n in dir(abi) if n.startswith("GT_") and isinstance(getattr(abi, n), int)]
    lines = ['#include <stdio.h>', f'#include "{HEADER}"', "int main(void){"]
    lines += [f'printf("{n} %llu\\n", (unsigned long long)({n}));' for n in names]
    lines.append("return 0;}")
    src = tmp_path / "consts.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "consts"
    subprocess.run(["gcc", "-std=c99", str(src), "-o", str(exe)], check=True)
    got = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                               check=True).stdout.splitlines())
    assert len(names) > 20
    for n in names:
        assert int(got[n]) == getattr(abi, n) & 0xFFFFFFFFFFFFFFFF, n


def test_camera_defaults_match_ray_camera_new():
    # RayCamera::new (graphics/camera.rs:1034-1065).
    d = abi.gt_camera_desc()
    assert lib().gt_camera_default(400, 16.0 / 9.0, C.byref(d)) == abi.GT_OK
    assert (d.samples_per_pixel, d.max_depth, d.russian_roulette_min_depth, d.rng_seed) == (1, 10, 5, 1)
    assert d.vertical_fov == 90.0 and list(d.lookat) == [0.0, 0.0, -1.0] and list(d.view_up) == [0.0, 1.0, 0.0]
    assert list(d.background)[:3] == [0.70, 0.80, 1.00] and d.light_pdf_weight == 0.5
    w, h, s = C.c_uint32(), C.c_uint32(), C.c_uint32()
    assert lib().gt_camera_image_size(C.byref(d), C.byref(w), C.byref(h), C.byref(s)) == abi.GT_OK
    assert (w.value, h.value, s.value) == (400, 225, 1)


def test_python_camera_defaults_equal_the_library_defaults():
    # RayCamera() describes a camera without the device library; its fields equal
    # gt_camera_default's byte for byte.
    from gartus_gb300.raytracing import RayCamera
    for w, aspect in ((400, 16.0 / 9.0), (1, 1.0), (600, 1.0)):
        d = abi.gt_camera_desc()
        assert lib().gt_camera_default(w, aspect, C.byref(d)) == abi.GT_OK
        assert bytes(RayCamera(w, aspect).desc()) == bytes(d)


def test_invalid_camera_is_rejected_without_a_device():
    # validate_view (camera.rs:1161-1201) panics; the ABI returns GT_ERR_INVALID_ARG.
    d = abi.gt_camera_desc()
    lib().gt_camera_default(8, 1.0, C.byref(d))
    d.vertical_fov = 180.0
    w = C.c_uint32()
    assert lib().gt_camera_image_size(C.byref(d), C.byref(w), None, None) == abi.GT_ERR_INVALID_ARG
    assert b"field of view" in lib().gt_last_error()
    lib().gt_camera_default(8, 1.0, C.byref(d))
    d.lookat[:] = list(d.lookfrom)
    assert lib().gt_camera_image_size(C.byref(d), C.byref(w), None, None) == abi.GT_ERR_INVALID_ARG
    assert lib().gt_camera_default(0, 1.0, C.byref(d)) == abi.GT_ERR_INVALID_ARG


def test_stratified_sample_counts():
    # effective_samples_per_pixel (camera.rs:1547-1556).
    from gartus_gb300.raytracing import RayCamera
    assert RayCamera(4, 1.0).with_samples_per_pixel(10).with_stratified_sampling().image_size()[2] == 9
    assert RayCamera(4, 1.0).with_stratified_grid_width(16).image_size()[2] == 256
    assert RayCamera(600, 1.0).image_size()[:2] == (600, 600)
    assert RayCamera(400, 16.0 / 9.0).image_size()[:2] == (400, 225)


def test_no_context_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from gartus_gb300.raytracing import Context
    with pytest.raises(GartusError):
        Context(0)
