"""Parameter files (.par) and the benchmark cases of the NuSiF hot path.

``write_par`` emits files in the reference's format (src/parameter.c:32-98,
dcavity.par, canal.par). Every value is followed by a comment so that the
reference parser, which splits on spaces only, never keeps a trailing newline
inside a value (a ``name`` ending in a newline silently disables the special
boundary condition in the reference).
"""
from __future__ import annotations

from pathlib import Path

# values of the reference's dcavity.par fixture
DCAVITY = {
    "name": "dcavity",
    "bcLeft": 1, "bcRight": 1, "bcBottom": 1, "bcTop": 1, "bcFront": 1, "bcBack": 1,
    "gx": 0.0, "gy": 0.0, "gz": 0.0,
    "re": 1000.0,
    "u_init": 0.0, "v_init": 0.0, "w_init": 0.0, "p_init": 0.0,
    "xlength": 1.0, "ylength": 1.0, "zlength": 1.0,
    "imax": 128, "jmax": 128, "kmax": 128,
    "te": 10.0, "dt": 0.02, "tau": 0.5,
    "levels": 2, "presmooth": 50, "postsmooth": 5,
    "itermax": 1000, "eps": 0.001, "omg": 1.8, "gamma": 0.9,
}

# values of the reference's canal.par fixture
CANAL = dict(DCAVITY, **{
    "name": "canal", "bcLeft": 3, "bcRight": 3, "re": 100.0, "u_init": 1.0,
    "xlength": 30.0, "ylength": 4.0, "zlength": 4.0, "imax": 200, "jmax": 40, "kmax": 40,
    "te": 60.0, "levels": 1, "itermax": 500, "eps": 0.0001,
})


def _fmt(v) -> str:
    if isinstance(v, float):
        return repr(v)
    return str(v)


def write_par(path: str | Path, values: dict, header: str = "generated case") -> Path:
    """Write ``values`` as a .par file (one ``key value # ...`` line each)."""
    path = Path(path)
    lines = [f"# {header}"]
    for k, v in values.items():
        lines.append(f"{k} {_fmt(v)}  #")
    path.write_text("\n".join(lines) + "\n")
    return path


def cavity(n: int | tuple[int, int, int], **over) -> dict:
    """Lid-driven cavity on the unit cube with ``n`` cells per axis."""
    i, j, k = (n, n, n) if isinstance(n, int) else n
    return dict(DCAVITY, imax=i, jmax=j, kmax=k, **over)


def config1(**over) -> dict:
    """64^3 cavity, Re 1000, tau 0.5 to t=1.0, RB-SOR omega 1.7, eps 1e-3, itermax 500."""
    return cavity(64, re=1000.0, tau=0.5, te=1.0, omg=1.7, eps=1e-3, itermax=500,
                  gamma=0.9, **over)


def config2(solver: str = "rb", **over) -> dict:
    """256^3 cavity, Re 1000, tau 0.5; RB (omega 1.7, eps 1e-6, itermax 10000) or MG."""
    base = cavity(256, re=1000.0, tau=0.5, te=1e9, omg=1.7, eps=1e-6, itermax=10000,
                  gamma=0.9, solver=solver, rtol=1e-6, mg_pre=2, mg_post=2)
    base.update(over)
    return base


def channel(**over) -> dict:
    """4x1x1 channel, 512x128x128, inflow 1 at x=0, outflow at x=4, Re 100."""
    base = dict(DCAVITY, name="canal", bcLeft=3, bcRight=3, re=100.0,
                xlength=4.0, ylength=1.0, zlength=1.0, imax=512, jmax=128, kmax=128,
                te=1e9, tau=0.5, inflow=1.0, solver="mg-mixed", rtol=1e-8)
    base.update(over)
    return base
