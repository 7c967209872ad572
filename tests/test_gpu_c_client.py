"""The C ABI from plain C, no Python in the loop: ``tests/c_client/pf_client.c``
is compiled with nvcc against the in-tree ``libpfgb300.so`` and runs K steps
of ``pfg_pf_step`` on parameters, eta and T written here; its eta must equal
the Python drop-in's (``PFSolver.stepper``) bit for bit on the same inputs."""
import os
import subprocess

import numpy as np
import pytest
import torch

from tests.cases import pf_case

pytestmark = pytest.mark.gpu


def test_c_client_matches_python_drop_in(tmp_path):
    from jax_am_gb300 import _build
    from jax_am_gb300.phase_field.allen_cahn import PFSolver, make_pf_params
    lib_path = _build.build()
    lib_dir = os.path.dirname(lib_path)
    exe = str(tmp_path / "pf_client")
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "c_client", "pf_client.c")
    r = subprocess.run([_build.nvcc_path(), "-o", exe, src, "-I", _build.INCLUDE, "-L", lib_dir,
                        "-lpfgb300", "-Xlinker", "-rpath," + lib_dir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr

    poly, eta, T, pf_args, _, _ = pf_case((37, 21, 9), 20, 0.15, seed=4)
    params = make_pf_params(pf_args, poly)
    files = {k: str(tmp_path / f"{k}.bin") for k in ("params", "eta0", "T", "out")}
    with open(files["params"], "wb") as f:
        f.write(bytes(params))
    np.ascontiguousarray(eta, dtype=np.float32).tofile(files["eta0"])
    np.ascontiguousarray(T, dtype=np.float32).reshape(-1).tofile(files["T"])
    steps, dt = 5, float(np.float32(1e-8))
    r = subprocess.run([exe, files["params"], files["eta0"], files["T"], str(steps), repr(dt),
                        files["out"]], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    got = np.fromfile(files["out"], dtype=np.float32).reshape(eta.shape)

    s = PFSolver(pf_args, poly)
    state = (torch.tensor(eta, dtype=torch.float32, device="cuda"), 0.0)
    Td = torch.tensor(T, dtype=torch.float32, device="cuda")
    t = 0.0
    for _ in range(steps):
        state, _ = s.stepper(state, t + dt, [Td])
        t = state[1]
    ref = state[0].cpu().numpy()
    assert np.array_equal(got, ref), float(np.abs(got - ref).max())
