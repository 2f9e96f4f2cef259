"""The C++ node layer: zeno's CuLagrange MPM node names, sockets, parameter
names and defaults, checked against the reference's ZENDEFNODE declarations
(tests/golden/reference_node_descriptors.json, made by
make_reference_descriptors.py from the reference sources)."""
import json
import os

import numpy as np
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
    zeno_inc = os.environ.get("ZENO_INCLUDE") or (
        os.path.join(REF_DEFAULT, "zeno", "include") if REF_DEFAULT else None)
    if not zeno_inc or not os.path.isdir(zeno_inc):
        pytest.skip("zeno headers not given (ZENO_INCLUDE or ZENO_REFERENCE)")
    root = os.path.dirname(HERE)
    cxx = shutil.which("g++") or "g++"
    r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-DZSMPM_WITH_ZENO", "-I", zeno_inc,
                        "-I", os.path.join(root, "include"),
                        os.path.join(root, "zeno_gb300", "nodes", "MPMNodes.cpp")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


# ConfigConstitutiveModel's meaning, not only its sockets: the "params" dict
# (Generation.cu:32,53-58) is read where the reference reads it.
MPM_FCR, MPM_NHK, MPM_STVK, MPM_EOS = 0, 1, 2, 3
MPM_PLASTIC_NONE, MPM_PLASTIC_NADP = 0, 1


def test_config_model_reads_friction_angle_from_params(zsmpm_mod):
    m, vol = zsmpm_mod.config_model("stvk", "nadp", E=1e5, nu=0.3, dx=1.0 / 256, ppc=8.0,
                                    params={"friction_angle": 30.0})
    assert m["plasticity"] == MPM_PLASTIC_NADP and m["type"] == MPM_STVK
    assert m["friction_angle_deg"] == 30.0
    assert vol == np.float32((1.0 / 256) ** 3 / 8.0)
    # no params: the reference default of 35 degrees (Generation.cu:70)
    m, _ = zsmpm_mod.config_model("fcr", "nadp", E=1e5, nu=0.3)
    assert m["friction_angle_deg"] == 35.0 and m["type"] == MPM_STVK


def test_config_model_params_of_other_models(zsmpm_mod):
    # the fluid extension takes its bulk modulus and exponent from params
    m, _ = zsmpm_mod.config_model("eos", "none", params={"bulk": 2e4, "gamma": 5.0})
    assert m["type"] == MPM_EOS and m["bulk"] == 2e4 and m["gamma"] == 5.0
    m, _ = zsmpm_mod.config_model("nhk", "none", E=5e4, nu=0.3, params={"friction_angle": 20.0})
    assert m["type"] == MPM_NHK and m["plasticity"] == MPM_PLASTIC_NONE
    assert m["E"] == 5e4 and m["nu"] == np.float32(0.3)


def test_config_model_rejects_unknown_model(zsmpm_mod):
    with pytest.raises(RuntimeError, match="unrecognized"):
        zsmpm_mod.config_model("bogus")
