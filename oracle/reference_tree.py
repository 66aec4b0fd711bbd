"""Where the reference renderer's source tree lies, for the oracle's build recipe.

TEST INFRASTRUCTURE, part of the recipe that compiles the reference's own shader
functions and importers into oracle/_ref/ (oracle/Makefile, target `ref`). The tree
is found from LUZ_REF_ROOT, else from the read-only mount of the build container
(the Makefile's default). Where neither holds the tree — on a machine that only
runs the prebuilt files — `reference_root()` returns None and the recipe and the
pin tests that need the tree are skipped.
"""
from __future__ import annotations

import os

DEFAULT_MOUNT = "/root/reference"


def reference_root() -> str | None:
    root = os.environ.get("LUZ_REF_ROOT") or DEFAULT_MOUNT
    return root if os.path.isdir(os.path.join(root, "source", "Shaders")) else None
