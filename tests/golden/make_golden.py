"""Generates tests/golden/reference_tables.json from the reference's source text.

The reference ships no tests or fixtures for the DFSPH path; its only pinned
numbers are data tables and constants in the source. This script reads them
(as text; nothing is compiled or run) from a VFD checkout and writes a small
fixture that the oracle and the CUDA library are checked against:

  * the surface-tension direction table haltonVec (HaltonVec323.cuh:4) as
    float32: its SHA-256 and a strided sample;
  * the 16-point Gauss-Legendre rule the volume map uses (p = 30,
    Core/Math/GaussQuadrature.cpp: GaussianN1, GaussianAbscissae1, GaussianWeights1);
  * the surface-tension classifier constants (DFSPHImplementation.cu:360-365);
  * the description defaults (DFSPHSimulationDescription.h:11-48);
  * the scene-file layout: the component order of Scene::Save (Scene/Scene.cpp:17-30)
    and the archive names of the DFSPH description, rigid-body and fluid-object
    serializers (Scene/Components/*.h), as the scene loader reads them.

Usage: python tests/golden/make_golden.py VFD_ROOT
(the root of a VFD checkout). Run only where the reference is present.
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _array_body(text: str, start_pattern: str) -> str:
    i = text.index(start_pattern)
    j = text.index("{", i)
    depth, k = 0, j
    while True:
        c = text[k]
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                return text[j + 1:k]
        k += 1


NUM = re.compile(r"[-+]?\d+\.?\d*(?:[eE][-+]?\d+)?")


def halton(root: str) -> dict:
    path = os.path.join(root, "VFD/Source/Simulation/DFSPH/HaltonVec323.cuh")
    body = _array_body(open(path).read(), "haltonVec[]")
    vals = np.array([float(t) for t in NUM.findall(body)], dtype=np.float64).astype(np.float32)
    assert vals.size == 49152, vals.size
    idx = list(range(0, 49152, 997)) + list(range(24))
    return dict(count=int(vals.size), sha256=hashlib.sha256(vals.tobytes()).hexdigest(),
                sample_index=idx, sample=[float(vals[i]) for i in idx])


def gauss_legendre(root: str, p: int = 30) -> dict:
    text = open(os.path.join(root, "VFD/Source/Core/Math/GaussQuadrature.cpp")).read()
    n_body = _array_body(text, "GaussianN1[")
    counts = [int(t) for t in re.findall(r"\b\d+\b", re.sub(r"//[^\n]*", "", n_body))]
    n = counts[p]

    def table(name: str) -> list[float]:
        body = _array_body(text, name)
        blocks = re.split(r"//\s*p\s*=\s*(\d+)", body)
        for k in range(1, len(blocks), 2):
            if int(blocks[k]) == p:
                return [float(t) for t in NUM.findall(blocks[k + 1])][:n]
        raise KeyError(p)

    return dict(p=p, n=n, abscissae=table("GaussianAbscissae1["), weights=table("GaussianWeights1["))


def constants(root: str) -> dict:
    text = open(os.path.join(root, "VFD/Source/Simulation/DFSPH/DFSPHImplementation.cu")).read()
    out = {}
    for name in ("ClassifierSlope", "ClassifierConstant", "SmoothingFactor", "Factor"):
        m = re.search(r"m_Info\." + name + r"\s*=\s*(" + NUM.pattern + r")f?;", text)
        out[name] = float(m.group(1))
    m = re.search(r"m_Info\.Volume\s*=\s*(" + NUM.pattern + r")f?\s*\*", text)
    out["VolumeFactor"] = float(m.group(1))
    m = re.search(r"m_Info\.Density0\s*=\s*(" + NUM.pattern + r")f?;", text)
    out["Density0"] = float(m.group(1))
    return out


def defaults(root: str) -> dict:
    text = open(os.path.join(root, "VFD/Source/Simulation/DFSPH/Structures/DFSPHSimulationDescription.h")).read()
    body = text[text.index("struct DFSPHSimulationDescription"):text.index("inline bool operator==")]
    out = {}
    for m in re.finditer(r"(\w+)\s+(\w+)\s*=\s*([^;]+);", body):
        typ, name, val = m.group(1), m.group(2), m.group(3).strip()
        if typ == "bool":
            out[name] = 1 if val == "true" else 0
        elif name == "Gravity":
            out[name] = [float(t) for t in NUM.findall(val)]
        else:
            out[name] = float(NUM.findall(val)[0])
    return out


def scene_format(root: str) -> dict:
    src = os.path.join(root, "VFD", "Source", "Scene")
    with open(os.path.join(src, "Scene.cpp")) as f:
        text = f.read()
    m = re.search(r"entt::snapshot\s*\{[^}]*\}\s*\.entities\(output\)\s*\.component<([^>]*)>", text)
    order = [t.strip() for t in m.group(1).split(",")]

    def nvps(name: str) -> list[str]:
        with open(os.path.join(src, "Components", name)) as f:
            return re.findall(r'make_nvp\("([^"]+)"', f.read())

    return dict(components=order, dfsph_description=nvps("DFSPHSimulationComponent.h"),
                rigid_body=nvps("RigidBodyComponent.h"), fluid_object=nvps("FluidObjectComponent.h"),
                transform=nvps("TransformComponent.h"), mesh=nvps("MeshComponent.h"))


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py VFD_ROOT")
    root = sys.argv[1]
    data = dict(source="VFD (Goubermouche/VFD) source text", halton=halton(root), gauss_legendre=gauss_legendre(root),
                constants=constants(root), description_defaults=defaults(root), scene_format=scene_format(root))
    out = os.path.join(HERE, "reference_tables.json")
    with open(out, "w") as f:
        json.dump(data, f, indent=1)
    print("wrote", out)


if __name__ == "__main__":
    main()
