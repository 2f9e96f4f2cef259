"""The node layer inside a real zeno core: zeno/src compiled from a
zenustech/zeno checkout (ZENO_REFERENCE; skipped without it), the node file
compiled against zeno's own headers into a plugin, and a host program that
loads both (tests/zeno_host/).  Checks that every reference MPM node is
registered in zeno's Session with the reference's sockets and defaults, and
that ConfigConstitutiveModel, run through zeno's own Graph with a "params"
DictObject, makes the material the reference would.  CPU only: the nodes
that launch substeps need a GPU, and the GPU host has no zeno checkout."""
import json
import os
import subprocess

import pytest

from .test_nodes import EXTENDED_ENUMS, EXTRA_INPUTS

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def host_output(zsmpm_mod):
    from .golden.make_reference_descriptors import REF_DEFAULT
    if not REF_DEFAULT:
        pytest.skip("no zeno checkout (ZENO_REFERENCE)")
    from .zeno_host.build_zeno_host import build
    out = build(REF_DEFAULT)
    r = subprocess.run([out["host"]], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l[len("ZSMPM_HOST "):] for l in r.stdout.splitlines() if l.startswith("ZSMPM_HOST ")]
    return json.loads(lines[0]), [json.loads(l) for l in lines[1:]]


def test_nodes_registered_in_zeno_session(host_output):
    descriptors, _ = host_output
    with open(os.path.join(HERE, "golden", "reference_node_descriptors.json")) as f:
        reference = json.load(f)
    assert set(reference) <= set(descriptors), sorted(set(reference) - set(descriptors))
    for node, ref in reference.items():
        for kind in ("inputs", "outputs", "params"):
            mine = {s[1]: s for s in descriptors[node][kind]}
            for typ, name, defl in ref[kind]:
                assert name in mine, (node, kind, name)
                mtyp, _, mdefl = mine[name]
                if (node, name) in EXTENDED_ENUMS:
                    assert set(typ.split()) <= set(mtyp.split()), (node, name)
                else:
                    assert mtyp == typ, (node, name, typ, mtyp)
                assert mdefl == defl, (node, name, defl, mdefl)
            # zeno's Descriptor appends an "SRC" input and a "DST" output to
            # every node (zeno/src/core/Descriptor.cpp)
            extra = set(mine) - {s[1] for s in ref[kind]} - {"SRC", "DST"}
            if kind == "inputs":
                assert extra <= EXTRA_INPUTS.get(node, set()), (node, extra)
            else:
                assert not extra, (node, kind, extra)
        assert descriptors[node]["categories"] == ref["categories"]
    # zeno's own nodes are there too: a real session, not the mirror
    assert "BeginFor" in descriptors and "MakeDict" in descriptors


def test_config_model_through_zeno_graph(host_output):
    _, models = host_output
    sand30, sand_default, snhk = models
    assert sand30["model"] == 1 and sand30["type"] == 2 and sand30["plasticity"] == 1
    assert sand30["friction_angle_deg"] == 30.0  # params={friction_angle: 30}
    assert sand_default["friction_angle_deg"] == 35.0  # Generation.cu:70
    assert snhk["type"] == 4 and snhk["plasticity"] == 0
    assert abs(sand30["volume"] - (1.0 / 256) ** 3 / 8) < 1e-15
