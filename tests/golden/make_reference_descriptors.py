"""Extract the ZENDEFNODE descriptors of the reference MPM nodes.

Reads the reference sources (a zenustech/zeno checkout, given as the first
argument or by the ZENO_REFERENCE environment variable) and writes
reference_node_descriptors.json next to this script: {node: {"inputs":
[[type, name, default], ...], "outputs": ..., "params": ..., "categories":
[...]}}.  Run once where the reference is present; the JSON is the committed
fixture the node tests compare against.
"""
import json
import os
import re
import sys

# the zeno checkout to read, or None (then the scripts and tests that need
# it are skipped)
REF_DEFAULT = os.environ.get("ZENO_REFERENCE")
FILES = ["projects/CuLagrange/mpm/Generation.cu", "projects/CuLagrange/mpm/Generation.cpp",
         "projects/CuLagrange/mpm/MPMPipeline.cu", "projects/CuLagrange/mpm/Transfer.cu",
         "projects/CuLagrange/mpm/Boundary.cu", "projects/CuLagrange/mpm/Temp.cu"]
NODES = ["ConfigConstitutiveModel", "ToZSParticles", "MakeZSPartition", "MakeZSGrid",
         "ZSPartitionForZSParticles", "ExpandZSPartition", "ZSGridFromZSPartition",
         "ZSParticleToZSGrid", "UpdateZSGrid", "ApplyBoundaryOnZSGrid", "ToZSBoundary",
         "ZSGridToZSParticle", "ZSReturnMapping", "AdjustParticleMaterial",
         "UpdatePrimitiveFromZSParticles", "ZSParticlesToPrimitiveObject", "MakeZSLevelSet",
         "StepZSBoundary", "ComputeParticleBeta", "ComputeVonMises", "ToZSCloth", "WriteZSParticles",
         "ConstructBendingSprings", "RetrievePrimitiveFromZSParticles",
         "ExtractPrimitiveFromZSParticles", "UpdatePrimitiveAttributesFromZSParticles",
         "UpdatePrimitiveAttrFromZSParticles",
         "ToTrackerParticles", "ToBoundaryParticles", "ZSBoundaryPrimitiveToZSGrid",
         "ApplyGridBoundaryOnZSGrid"]


def parse_braces(s, i):
    """Parse a {...} initializer of strings starting at s[i] == '{'."""
    assert s[i] == "{"
    out, i = [], i + 1
    while True:
        while s[i] in " \t\r\n,":
            i += 1
        if s[i] == "}":
            return out, i + 1
        if s[i] == "{":
            v, i = parse_braces(s, i)
            out.append(v)
        elif s[i] == '"':
            j = s.index('"', i + 1)
            out.append(s[i + 1:j])
            i = j + 1
        else:
            raise ValueError(f"unexpected {s[i:i + 20]!r}")


def socket(x):
    if isinstance(x, str):
        return ["", x, ""]
    return [x[0], x[1], x[2] if len(x) > 2 else ""]


def main():
    REF = sys.argv[1] if len(sys.argv) > 1 else REF_DEFAULT
    if not REF:
        sys.exit("give the zeno checkout as the first argument or in ZENO_REFERENCE")
    found = {}
    for f in FILES:
        src = open(os.path.join(REF, f)).read()
        src = re.sub(r"//[^\n]*", "", src)
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"ZENDEFNODE\(\s*(\w+)\s*,", src):
            name = m.group(1)
            if name not in NODES:
                continue
            i = src.index("{", m.end())
            d, _ = parse_braces(src, i)
            found[name] = {"inputs": [socket(x) for x in d[0]],
                           "outputs": [socket(x) for x in d[1]],
                           "params": [socket(x) for x in d[2]],
                           "categories": d[3], "file": f}
    missing = set(NODES) - set(found)
    if missing:
        raise SystemExit(f"not found: {sorted(missing)}")
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)),
                       "reference_node_descriptors.json")
    with open(out, "w") as fh:
        json.dump(found, fh, indent=1, sort_keys=True)
    print(f"wrote {len(found)} descriptors to {out}")


if __name__ == "__main__":
    main()
