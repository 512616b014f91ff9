"""Where the reference checkout is, for test infrastructure that reads it.

The checkout's location comes from the SGLD_REFERENCE environment variable,
or else from oracle/_ref/REFERENCE_ROOT, which oracle/build_ref.sh writes when
it compiles the reference's kernels.  Returns None when neither names an
existing directory (for example on a machine without the checkout): callers
skip or fail with a message then.
"""
from __future__ import annotations

import os

HERE = os.path.dirname(os.path.abspath(__file__))
RECORD = os.path.join(HERE, "_ref", "REFERENCE_ROOT")


def reference_root() -> str | None:
    root = os.environ.get("SGLD_REFERENCE")
    if not root and os.path.exists(RECORD):
        with open(RECORD) as f:
            root = f.read().strip()
    return root if root and os.path.isdir(root) else None
