"""Grain statistics of a phase-field solution on the GPU.

The reference finds grains after a run (``jax_am/phase_field/utils.py:
181-310``, ``process_eta``): face-adjacent solid cells (T < T_liquidus) of the
same argmax orientation form a grain; grains are listed by orientation, then
in order of their smallest cell index; each grain gets its volume and the PCA
aspect ratio ``2 l0 / (l1 + l2)`` (``l`` = square roots of the explained
variances of its volume-weighted cell centres, descending), or 1 when it has
fewer than 5 cells.

``segment_grains`` runs the connected-component labelling and the per-grain
moment sums on the GPU (``pfg_grains``); the volumes and aspect ratios follow
on the host from each grain's exact integer moments (one 3 x 3 eigenproblem
per grain).  ``process_eta`` is the drop-in for the reference function,
reading the solution that ``PFSolver.write_sols`` wrote.

A collinear grain (all cells on one line) has two zero variances: its
aspect ratio is ``inf`` here, where the reference's floating-point PCA may
return a huge finite number instead.
"""
import ctypes
import os

import numpy as np
import torch

from .. import _lib
from .allen_cahn import as_device_f32, make_pf_params


class _Box:
    """What make_pf_params reads from a polycrystal, for a grid without one."""

    def __init__(self, h, n):
        self.mesh_h_xyz = h
        self.unique_grain_directions = np.zeros((3, n, 3))


def _cell_size(pf_args):
    if all(k in pf_args for k in ("domain_x", "domain_y", "domain_z")):
        return (pf_args["domain_x"] / pf_args["Nx"], pf_args["domain_y"] / pf_args["Ny"],
                pf_args["domain_z"] / pf_args["Nz"])
    h = pf_args.get("h", 1.0)
    return tuple(h) if not np.isscalar(h) else (h, h, h)


def _cell_volume(pf_args):
    """The reference's uniform cell volume domain_vol / N (utils.py:204-205)."""
    N = int(pf_args["Nx"]) * int(pf_args["Ny"]) * int(pf_args["Nz"])
    if all(k in pf_args for k in ("domain_x", "domain_y", "domain_z")):
        return pf_args["domain_x"] * pf_args["domain_y"] * pf_args["domain_z"] / N
    hx, hy, hz = _cell_size(pf_args)
    return hx * hy * hz


def aspect_ratios(records):
    """Aspect ratios from the grains' integer moments: the covariance of
    the cell centres (ddof = 1, exact integer numerators), its eigenvalues in
    descending order, 2 sqrt(ev0) / (sqrt(ev1) + sqrt(ev2)); 1 below 5 cells
    (utils.py:286-310).  Cell-centre scaling (h, the volume weights) cancels."""
    K = len(records)
    ar = np.ones(K)
    big = [k for k in range(K) if records[k][0] >= 5]
    if not big:
        return ar
    cov = np.zeros((len(big), 3, 3))
    pairs = ((0, 0, 0), (1, 1, 1), (2, 2, 2), (0, 1, 3), (0, 2, 4), (1, 2, 5))
    for j, k in enumerate(big):
        c, s, s2 = records[k]
        c = int(c)
        den = c * (c - 1)
        for a, b, m in pairs:
            # exact: (c * sum(ab) - sum(a) sum(b)) / (c (c - 1)), big Python ints
            v = (c * int(s2[m]) - int(s[a]) * int(s[b])) / den
            cov[j, a, b] = cov[j, b, a] = v
    ev = np.linalg.eigvalsh(cov)[:, ::-1]
    ln = np.sqrt(np.maximum(ev, 0.0))
    with np.errstate(divide="ignore", invalid="ignore"):
        ar[big] = 2.0 * ln[:, 0] / (ln[:, 1] + ln[:, 2])
    return ar


def segment_grains(pf_args, ori_inds, T, T_ghosted=False, max_grains=None):
    """Grains of an orientation map.

    ``ori_inds``: (N,) orientation index per cell (the argmax of eta);
    ``T``: (N,) or (N, 1) per-cell temperature, or the ghosted heat state with
    ``T_ghosted``.  Returns a dict with ``labels`` ((N,) int32 CUDA tensor,
    grain number in the reference's order, -1 in liquid), ``ori``,
    ``first_cell``, ``cells``, ``volumes`` and ``aspect_ratios`` (NumPy, one
    entry per grain in the reference's order)."""
    lib = _lib.load()
    N = int(pf_args["Nx"]) * int(pf_args["Ny"]) * int(pf_args["Nz"])
    ori = torch.as_tensor(np.asarray(ori_inds) if not torch.is_tensor(ori_inds) else ori_inds)
    ori = ori.to("cuda", torch.int32).reshape(-1).contiguous()
    if ori.numel() != N:
        raise ValueError(f"ori_inds has {ori.numel()} entries, expected {N}")
    n = int(ori.max().item()) + 1 if N else 1
    n = max(n, int(pf_args.get("num_oris", n)))
    args = dict(pf_args, num_oris=min(n, _lib.MAX_ORIS))
    for key, default in (("gas_const", 8.3), ("Qg", 1.4e5), ("L0", 3.5e3), ("kappa_g", 2.77e-6),
                         ("m_g", 2.4e5), ("anisotropy", 0.0), ("ad_hoc", 1.0)):
        args.setdefault(key, default)
    params = make_pf_params(args, _Box(_cell_size(pf_args), args["num_oris"]))
    T = as_device_f32(T, None, "T").reshape(-1)
    expect = (N if not T_ghosted else
              (int(pf_args["Nx"]) + 2) * (int(pf_args["Ny"]) + 2) * (int(pf_args["Nz"]) + 2))
    if T.numel() != expect:
        raise ValueError(f"T has {T.numel()} entries, expected {expect}")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    nbytes = int(lib.pfg_grain_scratch_bytes(ctypes.byref(params)))
    scratch = torch.empty(max(nbytes, 16), dtype=torch.uint8, device="cuda")
    count = torch.zeros(1, dtype=torch.int64, device="cuda")
    labels = torch.empty(N, dtype=torch.int32, device="cuda")
    rec = ctypes.sizeof(_lib.Grain)
    cap = int(max_grains) if max_grains else max(1024, N // 64)
    while True:
        buf = torch.empty(max(cap, 1) * rec // 8, dtype=torch.int64, device="cuda")
        st = lib.pfg_grains(ctypes.byref(params), _lib.ptr(ori), _lib.ptr(T), int(T_ghosted),
                            _lib.ptr(labels), _lib.ptr(buf), cap, _lib.ptr(count),
                            _lib.ptr(scratch), scratch.numel(), stream)
        _lib.check(st, "pfg_grains")
        K = int(count.item())
        if K <= cap:
            break
        cap = K
    raw = buf[: K * rec // 8].cpu().numpy().view(np.int64).reshape(K, rec // 8)
    # column 1 holds (ori, reserved) as two little-endian int32
    first, ori_g = raw[:, 0], (raw[:, 1] & 0xFFFFFFFF).astype(np.int64)
    cells, sums, sums2 = raw[:, 2], raw[:, 3:6], raw[:, 6:12]
    order = np.lexsort((first, ori_g))  # by orientation, then smallest cell index
    rank = np.empty(K, dtype=np.int64)
    rank[order] = np.arange(K)
    rank_t = torch.as_tensor(rank, dtype=torch.int32, device="cuda")
    lab = torch.where(labels >= 0, rank_t[labels.clamp(min=0).long()] if K else labels, labels)
    records = [(cells[k], sums[k], sums2[k]) for k in order]
    return {
        "labels": lab,
        "ori": ori_g[order].astype(np.int64),
        "first_cell": first[order],
        "cells": cells[order],
        "volumes": cells[order] * _cell_volume(pf_args),
        "aspect_ratios": aspect_ratios(records),
    }


def process_eta(pf_args, step=13):
    """Drop-in for the reference's ``process_eta`` (utils.py:181-214): reads
    the solution ``PFSolver.write_sols`` wrote for ``step`` (``<data_dir>/
    numpy/pf/sols/u<step>.npz``; the reference reads the VTU it wrote) and
    returns ``[grain volumes, grain aspect ratios]`` in the reference's grain
    order."""
    path = os.path.join(pf_args["data_dir"], f"numpy/pf/sols/u{step:03d}.npz")
    d = np.load(path)
    res = segment_grains(pf_args, d["ori_inds"], d["T"])
    return [list(res["volumes"]), list(res["aspect_ratios"])]
