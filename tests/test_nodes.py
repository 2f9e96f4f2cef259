"""The C++ node layer: zeno's CuLagrange MPM node names, sockets, parameter
names and defaults, checked against the reference's ZENDEFNODE declarations
(tests/golden/reference_node_descriptors.json, made by
make_reference_descriptors.py from the reference sources)."""
import json
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))

# sockets this backend adds to reference nodes (documented extensions)
EXTRA_INPUTS = {"ToZSBoundary": {"dx", "thickness", "domain_min", "domain_max"},
                # a ToZSCloth cloth and ToTrackerParticles points stepped with
                # the partitioned particles
                "ZSPartitionForZSParticles": {"ZSCloth", "ZSTrackers", "ZSBending"},
                # dense level sets filled from a primitive or an analytic shape
                "MakeZSLevelSet": {"sdf_prim", "dims", "shape", "center", "radius", "height",
                                   "extent"}}
# enum inputs whose option list this backend extends
EXTENDED_ENUMS = {("ConfigConstitutiveModel", "type")}


@pytest.fixture(scope="module")
def descriptors(zsmpm_mod):
    return zsmpm_mod.node_descriptors()


@pytest.fixture(scope="module")
def reference():
    with open(os.path.join(HERE, "golden", "reference_node_descriptors.json")) as f:
        return json.load(f)


def test_every_reference_node_is_registered(descriptors, reference):
    assert set(reference) <= set(descriptors), sorted(set(reference) - set(descriptors))


@pytest.mark.parametrize("kind", ["inputs", "outputs", "params"])
def test_sockets_match_reference(descriptors, reference, kind):
    for node, ref in reference.items():
        mine = {s[1]: s for s in descriptors[node][kind]}
        for typ, name, defl in ref[kind]:
            assert name in mine, f"{node}.{kind}: socket {name!r} missing"
            mtyp, _, mdefl = mine[name]
            if (node, name) in EXTENDED_ENUMS:
                assert set(typ.split()) <= set(mtyp.split()), (node, name, typ, mtyp)
            else:
                assert mtyp == typ, (node, name, typ, mtyp)
            assert mdefl == defl, (node, name, defl, mdefl)
        extra = set(mine) - {s[1] for s in ref[kind]}
        if kind == "inputs":
            assert extra <= EXTRA_INPUTS.get(node, set()), (node, extra)
        else:
            assert not extra, (node, kind, extra)
        assert descriptors[node]["categories"] == ref["categories"]


def test_fused_substep_node_registered(descriptors):
    d = descriptors["ZSMPMSubstep"]
    assert [s[1] for s in d["outputs"]] == ["ZSParticles", "MaxVelSqr"]


def test_node_file_compiles_against_zeno_headers():
    """The same MPMNodes.cpp compiles against zeno's own node API headers
    (inside zeno, ZSMPM_WITH_ZENO selects them instead of the mirror)."""
    import shutil
    import subprocess
    from .golden.make_reference_descriptors import REF_DEFAULT
    zeno_inc = os.environ.get("ZENO_INCLUDE", os.path.join(REF_DEFAULT, "zeno", "include"))
    if not os.path.isdir(zeno_inc):
        pytest.skip("zeno headers not present")
    root = os.path.dirname(HERE)
    cxx = shutil.which("g++") or "g++"
    r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-DZSMPM_WITH_ZENO", "-I", zeno_inc,
                        "-I", os.path.join(root, "include"),
                        os.path.join(root, "zeno_gb300", "nodes", "MPMNodes.cpp")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
