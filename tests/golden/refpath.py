"""Location of the reference checkout for the fixture generators.

The generators import the unmodified reference, so they need its source tree;
they take its path from the ``MCL_REFERENCE`` environment variable and stop
with a message when it is unset or wrong.  Nothing else in the repository
reads the reference: the tests use the fixtures these scripts wrote.
"""
from __future__ import annotations

import os
import sys


def reference_root() -> str:
    root = os.environ.get("MCL_REFERENCE", "")
    if not root or not os.path.isdir(os.path.join(root, "src", "class")):
        sys.exit("set MCL_REFERENCE to the root of a MCLuminescence checkout "
                 "(the directory that holds src/class/simulate.py)")
    return root
