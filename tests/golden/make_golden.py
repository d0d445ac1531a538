#!/usr/bin/env python3
"""Regenerate the golden fixtures in tests/golden/ from the reference tree.

The reference ships two FacetRT results produced by its Vulkan backend on
Windows (validation/<scene>/output/radiosity_gpu.json) next to the scene they
were computed on (radiosity_scene.obj, which the eFacetRT entry loads with
loadTreeWithSoil, facetrtcore.cpp:362-473).  This script copies each OBJ and
stores the per-side radiosity, sunlit and lightEnhancement vectors plus the
graph diagnostics as a compressed .npz, so the tests can run where the
reference tree is absent.

Usage: python tests/golden/make_golden.py [reference_root]
(default: the tree the oracle recipe reads, oracle/build_ref.py REFERENCE,
which FACETRT_REFERENCE_ROOT overrides)
"""
import json
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle.build_ref import REFERENCE  # noqa: E402

SCENES = ["urban_tree_building", "urban_dem_building"]


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else REFERENCE
    for scene in SCENES:
        out_dir = os.path.join(root, "validation", scene, "output")
        with open(os.path.join(out_dir, "radiosity_gpu.json"), encoding="utf-8") as f:
            result = json.load(f)
        shutil.copyfile(os.path.join(out_dir, "radiosity_scene.obj"),
                        os.path.join(HERE, f"{scene}.obj"))
        graph = result["graph"]
        np.savez_compressed(
            os.path.join(HERE, f"{scene}_vulkan.npz"),
            radiosity=np.asarray(result["radiosity"], np.float32),
            sunlit=np.asarray(result["sunlit"], np.float32),
            lightEnhancement=np.asarray(result["lightEnhancement"], np.float32),
            facetCount=np.int64(result["facetCount"]),
            leafFacetCount=np.int64(result["leafFacetCount"]),
            directedEdges=np.int64(graph["directedEdges"]),
            closureError=np.float64(graph["closureError"]),
            fragmentOverflow=np.int64(graph["fragmentOverflow"]),
            hashOverflow=np.int64(graph["hashOverflow"]),
            iterations=np.int64(result["iterations"]),
            timing=json.dumps(result["timing"]),
            backend=result["backend"],
        )
        print(scene, result["facetCount"], "facets")


if __name__ == "__main__":
    main()
