"""Generate ``tests/golden/point_sources.npz``: the reference drivers' own
analytic laser temperatures, evaluated at the cell centres of a small grid
by running their unmodified ``get_T_fn`` (and ``read_path``) under the
``jax`` stand-in of ``jax_standin.py`` (loaded with the stubs of
``make_golden.py``):

* ``applications/phase_field/simple/example.py:21-37`` at several times;
* ``applications/phase_field/simple/example_grf.py:21-46`` at several times;
* ``applications/phase_field/multi_scan/example.py:33-84`` at several steps
  of its sampled raster path.

Run from the repository root:
``python tests/golden/make_golden_point_sources.py --ref <reference tree>``
"""
import contextlib
import io
import os
import sys

import numpy as onp

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as MG  # noqa: E402  (installs the stand-in and the stubs)


class _Poly:
    pass


def main():
    Nx, Ny, Nz = 20, 12, 8
    dom = (2e-4, 1.2e-4, 0.8e-4)
    h = (dom[0] / Nx, dom[1] / Ny, dom[2] / Nz)
    zz, yy, xx = onp.meshgrid(onp.arange(Nz), onp.arange(Ny), onp.arange(Nx), indexing="ij")
    poly = _Poly()
    poly.centroids = onp.stack(((xx.ravel() + 0.5) * h[0], (yy.ravel() + 0.5) * h[1],
                                (zz.ravel() + 0.5) * h[2]), axis=1)
    args = dict(domain_x=dom[0], domain_y=dom[1], domain_z=dom[2], t_OFF=4e-4, T_ambient=300.0,
                vel=0.25, dt=2e-6,
                laser_path=dict(x_pos=[0.3e-4, 1.7e-4, 1.7e-4, 0.3e-4],
                                y_pos=[0.8e-4, 0.8e-4, 0.4e-4, 0.4e-4],
                                z_pos=[0.8e-4, 0.8e-4, 0.8e-4, 0.8e-4], switch=[1, 1, 0, 1]))
    simple = MG._load_example("applications/phase_field/simple/example.py")
    grf = MG._load_example("applications/phase_field/simple/example_grf.py")
    multi = MG._load_example("applications/phase_field/multi_scan/example.py")
    times = onp.array([0.0, 3.7e-5, 1.2e-4, 2.9e-4, 4.0e-4])
    T_simple = onp.stack([onp.asarray(simple.get_T_fn(poly, args)(t)) for t in times])
    T_grf = onp.stack([onp.asarray(grf.get_T_fn(poly, args)(t)) for t in times])
    with contextlib.redirect_stdout(io.StringIO()):
        ts, xs, ys, zs, ps, mov = multi.read_path(args)
    steps = onp.array([0, 17, 71, 140, len(ts) - 1])
    fn = multi.get_T_fn(poly, args)
    T_path = onp.stack([onp.asarray(fn(ts[i], xs[i], ys[i], zs[i], ps[i], mov[i])) for i in steps])
    onp.savez_compressed(os.path.join(HERE, "point_sources.npz"), shape=onp.array([Nx, Ny, Nz]),
                         domain=onp.array(dom), t_OFF=args["t_OFF"], T_ambient=args["T_ambient"],
                         vel=args["vel"], dt=args["dt"],
                         x_pos=args["laser_path"]["x_pos"], y_pos=args["laser_path"]["y_pos"],
                         z_pos=args["laser_path"]["z_pos"], switch=args["laser_path"]["switch"],
                         times=times, T_simple=T_simple, T_grf=T_grf, path_ts=ts, path_xs=xs,
                         path_ys=ys, path_zs=zs, path_ps=ps, path_dirs=mov, path_steps=steps,
                         T_path=T_path)
    print(f"{len(ts)} path samples; T ranges: simple {T_simple.min():.1f}..{T_simple.max():.1f}, "
          f"grf {T_grf.min():.1f}..{T_grf.max():.1f}, path {T_path.min():.1f}..{T_path.max():.1f}")


if __name__ == "__main__":
    main()
