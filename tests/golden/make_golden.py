"""Generates the golden fixtures under tests/golden/ (run: python tests/golden/make_golden.py,
or with the argument `operators` for ops_small.npz alone).

The reference (Fortran + MPI) cannot be built in this environment, so the expected outputs
are produced by the CPU oracle (oracle/lpm_oracle.c), itself pinned by the reference's PSE
regression thresholds and the mesh invariants (see tests/test_oracle.py).  The fixtures
freeze small inputs together with the oracle's outputs so that the GPU tests compare
against committed numbers and any change of the oracle is caught.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "lpm-v2_gb300"))

import lpm_gpu as lg  # noqa: E402
import workloads as wl  # noqa: E402
from oracle import oracle as orc  # noqa: E402

PI = wl.PI


def sphere_case(nest, seed):
    m = lg.PolyMesh2d(lg.ICOS_TRI_SPHERE_SEED, nest, 1.0)
    rng = np.random.default_rng(seed)
    c = wl.random_unit_vector(rng)
    zeta = wl.gaussian_vortex(m, 4.0 * PI, 32.0, c) + 0.5 * wl.rh54_vorticity(m)
    return m, zeta


def main():
    # ---- sphere BVE velocity + stream functions (icos nest 2, 482 particles)
    m, zeta = sphere_case(2, 1)
    x, y, z, a, act = m.x, m.y, m.z, m.area, m.active
    u, v, w = orc.bve_velocity(x, y, z, zeta, a, act, 1.0, orc.ASSOC_SOLVER)
    um, vm, wm = orc.bve_velocity(x, y, z, zeta, a, act, 1.0, orc.ASSOC_MESH)
    absv = zeta + 2.0 * (2.0 * PI) * z
    pr, pa = orc.bve_stream(x, y, z, zeta, absv, a, act, 1.0)
    # off-sphere positions (an RK4 stage input: x + dt/2 k) exercise the |x| != a terms
    xo, yo, zo = x + 0.005 * u, y + 0.005 * v, z + 0.005 * w
    uo, vo, wo = orc.bve_velocity(xo, yo, zo, zeta, a, act, 1.0, orc.ASSOC_SOLVER)
    np.savez(HERE / "bve_icos2.npz", x=x, y=y, z=z, zeta=zeta, area=a, active=act, u=u, v=v, w=w, um=um, vm=vm,
             wm=wm, absvort=absv, psi_rel=pr, psi_abs=pa, xo=xo, yo=yo, zo=zo, uo=uo, vo=vo, wo=wo)

    # ---- RK4 trajectory, 10 steps (icos nest 2)
    s = orc.bve_timestep(x, y, z, zeta, a, act, u, v, w, 1.0, 2.0 * PI, 0.01, 10)
    np.savez(HERE / "bve_rk4_icos2.npz", x0=x, y0=y, z0=z, zeta0=zeta, u0=u, v0=v, w0=w, area=a, active=act,
             x=s[0], y=s[1], z=s[2], zeta=s[3], u=s[4], v=s[5], w=s[6], dt=0.01, steps=10, omega=2.0 * PI)

    # ---- planar velocity + stream function (quad nest 3 on [-4, 4]^2, 289 particles)
    mp = lg.PolyMesh2d(lg.QUAD_RECT_SEED, 3, 4.0)
    om = wl.colliding_dipoles(mp.x, mp.y, width_sq=0.5)
    pu0, pv0 = orc.plane_velocity(mp.x, mp.y, om, mp.area, mp.active, 0.0)
    pu2, pv2 = orc.plane_velocity(mp.x, mp.y, om, mp.area, mp.active, 0.02)
    ps = orc.plane_stream(mp.x, mp.y, om, mp.area, mp.active)
    t = orc.plane_timestep(mp.x, mp.y, om, mp.area, mp.active, pu0, pv0, 0.0, 0.005, 10)
    np.savez(HERE / "plane_quad3.npz", x=mp.x, y=mp.y, omega=om, area=mp.area, active=mp.active, u0=pu0, v0=pv0,
             u2=pu2, v2=pv2, psi=ps, xs=t[0], ys=t[1], us=t[2], vs=t[3], dt=0.005, steps=10)

    # ---- PSE Laplacian (icos nest 2 sphere; quad nest 3 plane)
    rng = np.random.default_rng(0)
    f = wl.y54(x, y, z) + 1e-3 * rng.random(m.n)
    eps_k8 = m.max_edge_length ** 0.75
    eps_g = 2.0 * m.avg_edge_length
    lk = orc.pse_laplacian(x, y, z, f, a, act, eps_k8, 1.0, orc.PSE_K8_GEODESIC)
    lg_ = orc.pse_laplacian(x, y, z, f, a, act, eps_g, 1.0, orc.PSE_GAUSS_CHORD)
    fp = np.sin(mp.x) * np.cos(0.5 * mp.y)
    eps_p = mp.max_edge_length ** 0.75
    lp = orc.pse_laplacian(mp.x, mp.y, None, fp, mp.area, mp.active, eps_p, 1.0, orc.PSE_K8_CHORD)
    np.savez(HERE / "pse_small.npz", x=x, y=y, z=z, f=f, area=a, active=act, eps_k8=eps_k8, eps_g=eps_g,
             lap_k8=lk, lap_gauss=lg_, px=mp.x, py=mp.y, pf=fp, parea=mp.area, pactive=mp.active, peps=eps_p,
             plap=lp)
    print("wrote", sorted(p.name for p in HERE.glob("*.npz")))


def operators():
    """ops_small.npz: the other PSE operators, the SWE integrals and the beta plane, small."""
    out = {}
    # sphere: icos nest 2
    m, zeta = sphere_case(2, 2)
    x, y, z, a, act = m.x, m.y, m.z, m.area, m.active
    f = wl.y54(x, y, z)
    gx, gy, gz = wl.y54_surface_gradient(x, y, z)
    eps = m.max_edge_length ** 0.5
    out.update(sx=x, sy=y, sz=z, sa=a, sact=act, szeta=zeta, sf=f, sgx=gx, sgy=gy, sgz=gz, seps=eps)
    out["grad"] = np.stack(orc.pse_sphere_gradient(x, y, z, f, a, act, eps, 1.0))
    out["div"] = orc.pse_sphere_divergence(x, y, z, gx, gy, gz, a, act, eps, 1.0)
    out["sddot"] = orc.pse_sphere_double_dot(x, y, z, gx, gy, gz, a, act, eps, 1.0)
    q = np.stack([np.cos(np.linspace(0, 6, 16)), np.sin(np.linspace(0, 6, 16)), np.zeros(16)])
    out["sq"] = q
    out["sinterp"] = orc.pse_interpolate(x, y, z, f, a, act, eps, q[0], q[1], q[2], 1, 1.0)
    div = 0.1 * np.cos(3.0 * z)
    sh = 1.0 + 0.2 * z
    out.update(sdivv=div, ssh=sh)
    out["sswe"] = np.stack(orc.swe_sphere_rhs(x, y, z, zeta, div, sh, a, act, 1.0, 1.0, 0.25))
    # plane: quad nest 3 on [-4, 4]^2
    mp = lg.PolyMesh2d(lg.QUAD_RECT_SEED, 3, 4.0)
    px, py, pa, pact = mp.x, mp.y, mp.area, mp.active
    pf = np.sin(px) * np.cos(0.5 * py)
    peps = 2.0 * np.sqrt(pa[pact == 1].max())
    out.update(px=px, py=py, pa=pa, pact=pact, pf=pf, peps=peps)
    pg = orc.pse_plane_gradient(px, py, pf, pa, pact, peps)
    out["pgrad"] = np.stack(pg)
    out["psecond"] = np.stack(orc.pse_plane_second_partials(px, py, pg[0], pg[1], pa, pact, peps))
    out["pddot"] = orc.pse_plane_double_dot(px, py, pg[0], pg[1], pa, pact, peps)
    pq = np.stack([np.linspace(-3, 3, 16), np.linspace(2, -2, 16), np.zeros(16)])
    out["pq"] = pq
    out["pinterp"] = orc.pse_interpolate(px, py, None, pf, pa, pact, peps, pq[0], pq[1], None, 0, 1.0)
    vort = np.exp(-(px ** 2 + py ** 2))
    pdiv = 0.3 * np.exp(-((px - 1) ** 2 + py ** 2))
    psh = 1.0 + 0.1 * np.cos(px)
    out.update(pvort=vort, pdivv=pdiv, psh=psh)
    out["pswe"] = np.stack(orc.swe_plane_rhs(px, py, vort, pdiv, psh, pa, pact, peps))
    # beta plane: 300 random points on the strip
    rng = np.random.default_rng(3)
    bx, by = rng.random(300), rng.uniform(-0.5, 0.5, 300)
    ba = rng.uniform(0.5, 1.5, 300) / 300
    bz = np.sin(2 * PI * bx) * np.exp(-8 * by * by)
    bact = (rng.random(300) < 0.8).astype(np.int32)
    out.update(bx=bx, by=by, ba=ba, bzeta=bz, bact=bact)
    out["bvel"] = np.stack(orc.beta_plane_velocity(bx, by, bz, ba, bact))
    out["bstream"] = np.stack(orc.beta_plane_stream(bx, by, bz, bz + 3.0 * by, ba, bact))
    np.savez_compressed(HERE / "ops_small.npz", **out)
    print("wrote ops_small.npz")


if __name__ == "__main__":
    if sys.argv[1:] == ["operators"]:
        operators()
    else:
        main()
        operators()
