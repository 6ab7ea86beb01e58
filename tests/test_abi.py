"""The C-ABI library without a GPU: it builds, loads, exports every entry point
declared in include/vfd_dfsph.h and include/vfd_sph.h, its structs have the layout the Python mirror
assumes, and calls that need a device fail with a status code (no hang, no exit).
"""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import vfd_gb300
from vfd_gb300 import _abi, sph

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", h) for h in ("vfd_dfsph.h", "vfd_sph.h")]


def header_functions():
    text = "".join(open(h).read() for h in HEADERS)
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+(vfd_\w+)\s*\(", text, re.M)))


def test_python_mirror_lists_every_header_function():
    assert sorted(vfd_gb300.EXPORTS) == header_functions()


def test_library_exports_every_header_function(built_library):
    L = C.CDLL(built_library)
    missing = [f for f in header_functions() if not hasattr(L, f)]
    assert not missing, missing


def test_library_has_no_host_only_fallback(built_library):
    """The step entry points live in a library that links the CUDA runtime."""
    out = subprocess.run(["ldd", built_library], capture_output=True, text=True).stdout
    assert "libcudart" in out or "cudart" in open(built_library, "rb").read(2_000_000).decode("latin1")


def _c_layout(struct_name, fields):
    src = "#include <stdio.h>\n#include <stddef.h>\n#include \"vfd_sph.h\"\nint main(void){\n"
    src += f'printf("%zu\\n", sizeof({struct_name}));\n'
    for f in fields:
        src += f'printf("%zu\\n", offsetof({struct_name}, {f}));\n'
    src += "return 0;}\n"
    return src


@pytest.mark.parametrize("cls", [_abi.vfd_desc, _abi.vfd_volume_map, _abi.vfd_step_stats, _abi.vfd_info,
                                 _abi.vfd_adjoint_stats, sph.vfd_sph_desc, sph.vfd_sph_params])
def test_struct_layout_matches_header(tmp_path, cls):
    names = [n for n, _ in cls._fields_]
    src = tmp_path / "layout.c"
    src.write_text(_c_layout(cls.__name__, names))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert vals[0] == C.sizeof(cls)
    for (name, _), off in zip(cls._fields_, vals[1:]):
        assert getattr(cls, name).offset == off, name


def test_desc_default_matches_reference_defaults(built_library, golden):
    L = vfd_gb300.lib()
    d = _abi.vfd_desc()
    assert L.vfd_desc_default(C.byref(d)) == 0
    for k, v in golden["description_defaults"].items():
        got = getattr(d, k)
        if k == "Gravity":
            assert list(got) == pytest.approx(v)
        else:
            assert float(got) == pytest.approx(v, rel=1e-6), k


def test_abi_version(built_library):
    assert vfd_gb300.lib().vfd_abi_version() == 1


def test_box_map_sizes_match_oracle(built_library):
    from oracle import oracle as O
    for res in [(4, 5, 6), (20, 20, 20), (1, 1, 1)]:
        r = np.array(res, np.uint32)
        nn, nc = C.c_uint32(), C.c_uint32()
        assert vfd_gb300.lib().vfd_box_map_sizes(r.ctypes.data_as(C.POINTER(C.c_uint32)), C.byref(nn),
                                                 C.byref(nc)) == 0
        m = O.build_box_map((0, 0, 0), (1, 1, 1), True, 0.0, res, 0.1)
        assert nn.value == m.struct.node_count and nc.value == m.struct.cell_count


def test_argument_errors_are_status_codes(built_library):
    L = vfd_gb300.lib()
    assert L.vfd_create(None, None) == _abi.VFD_E_ARG
    assert L.vfd_step(None, None) == _abi.VFD_E_ARG
    req, act = C.c_int32(7), C.c_int32(7)
    assert L.vfd_get_graph_mode(None, C.byref(req), C.byref(act)) == _abi.VFD_E_ARG
    assert (req.value, act.value) == (7, 7)
    assert L.vfd_set_lanes(None, None, 0) == _abi.VFD_E_ARG
    assert L.vfd_destroy(None) == 0
    bad = _abi.make_desc(ParticleRadius=-1.0)
    h = C.c_void_p()
    assert L.vfd_create(C.byref(bad), C.byref(h)) == _abi.VFD_E_ARG
    assert b"ParticleRadius" in L.vfd_last_error()


def test_no_device_is_reported(built_library):
    """Without a GPU, creating a simulation returns VFD_E_NODEVICE instead of exiting."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(vfd_gb300.VFDError) as e:
        vfd_gb300.DFSPHSimulation()
    assert e.value.code == _abi.VFD_E_NODEVICE


def test_tuned_kernel_lists_agree():
    # vfd_set_lanes / vfd_autotune index lanes by the device's TunedKernel enum; the Python
    # names, the autotuner's kernel names and the header's documented order must follow it
    src = os.path.join(ROOT, "vfd_gb300", "csrc")
    enum = re.search(r"enum TunedKernel \{(.*?)\};", open(os.path.join(src, "dfsph_common.cuh")).read(), re.S).group(1)
    members = [m.strip().split("=")[0].strip() for m in enum.split(",") if m.strip()]
    assert members[-1] == "kTunedCount"
    assert len(members) - 1 == len(vfd_gb300.TUNED_KERNELS)
    api = open(os.path.join(src, "dfsph_api.cu")).read()
    names = re.search(r"names\[kTunedCount\] = \{(.*?)\};", api, re.S).group(1)
    names = re.findall(r'"(k_\w+)"', names)
    assert names == ["k_" + k for k in vfd_gb300.TUNED_KERNELS]
