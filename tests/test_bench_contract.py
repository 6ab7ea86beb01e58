"""bench.py's static parts, without a GPU: every kernel its roofline table names is a
kernel the library launches (by the name the per-kernel profiler reports), the default
run is the configuration's 500 steps with at least 3 warm-up steps, and the profiles'
per-particle traffic covers kernels of that table."""
import ast
import json
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench_tree():
    return ast.parse(open(os.path.join(ROOT, "bench.py")).read())


def _algo_bytes_keys():
    for node in ast.walk(_bench_tree()):
        if isinstance(node, ast.Assign) and any(getattr(t, "id", "") == "ALGO_BYTES" for t in node.targets):
            return [k.value for k in node.value.keys]
    raise AssertionError("ALGO_BYTES not found")


def _launched_names():
    names = set()
    src = os.path.join(ROOT, "vfd_gb300", "csrc")
    for f in os.listdir(src):
        if f.endswith((".cu", ".cuh")):
            text = open(os.path.join(src, f)).read()
            names.update(re.findall(r'(?:VFD|SEARCH)_LAUNCH(?:_MODE)?\((?:[A-Z_]+,\s*)?"(k_\w+)"', text))
            names.update(re.findall(r'VFD_TILE_DISPATCH\("(k_\w+)"', text))
    return names


def test_roofline_table_names_launched_kernels():
    launched = _launched_names()
    assert "k_cg_spmv" in launched and "k_neighbors" in launched
    stale = sorted(set(_algo_bytes_keys()) - launched)
    assert not stale, stale


def test_default_run_is_the_configuration():
    src = open(os.path.join(ROOT, "bench.py")).read()
    steps = int(re.search(r'"--steps", type=int, default=(\d+)', src).group(1))
    warm = int(re.search(r'"--warmup", type=int, default=(\d+)', src).group(1))
    assert steps == 500 and warm >= 3


def test_traffic_figures_cover_table_kernels():
    traffic = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
    keys = set(_algo_bytes_keys())
    for k, v in traffic.items():
        assert k in keys and v["bytes_per_particle"] > 0, k


def test_every_step_kernel_counts_its_launch():
    # gpu_launches is counted on the device: every kernel of the step increments the
    # launch counter (VFD_COUNT_LAUNCH) as its first statement
    src = os.path.join(ROOT, "vfd_gb300", "csrc")
    missing = []
    for f in ("dfsph_physics.cu", "dfsph_search.cu", "dfsph_boundary.cu"):
        text = open(os.path.join(src, f)).read()
        for m in re.finditer(r"__global__ void (?:__launch_bounds__\(\w+\) )?(k_\w+)\(Dev d\) \{", text):
            body = text[m.end():m.end() + 200]
            if "VFD_COUNT_LAUNCH(d)" not in body.split(";")[0] + ";":
                missing.append(m.group(1))
    assert not missing, missing


def test_device_code_has_no_trap_or_assert():
    # failures are reported through status words; no kernel traps or asserts on the device
    src = os.path.join(ROOT, "vfd_gb300", "csrc")
    for f in os.listdir(src):
        if f.endswith((".cu", ".cuh")):
            text = open(os.path.join(src, f)).read()
            assert "__trap" not in text, f
            assert not re.search(r"(?<!static_)\bassert\s*\(", text), f
