"""Where the golden-vector generators find the reference's source tree.

The tree is given by ``--ref PATH`` on the command line or by the
environment variable ``JAX_AM_REF``; with neither, the generators stop with
an error instead of guessing a machine path.
"""
import os
import sys


def reference_root():
    argv = sys.argv[1:]
    for i, a in enumerate(argv):
        if a == "--ref" and i + 1 < len(argv):
            root = argv[i + 1]
            break
        if a.startswith("--ref="):
            root = a.split("=", 1)[1]
            break
    else:
        root = os.environ.get("JAX_AM_REF")
    if not root:
        raise SystemExit("give the reference's source tree (the directory holding jax_am/ and "
                         "applications/) with --ref PATH or JAX_AM_REF=PATH")
    if not os.path.isdir(os.path.join(root, "jax_am")):
        raise SystemExit(f"{root!r} holds no jax_am/ directory")
    return os.path.abspath(root)
