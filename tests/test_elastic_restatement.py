"""A second, independent restatement of the reference's elastic step, written
with numpy slices straight from src/Core.jl:96-228 (fw1..fw4, one_step),
adbroadcast (src/Core.jl:679-695, including modes 3 / 4 returning their
input, so K is never applied), makevector (src/Core.jl:697-699: scatter into
a zero vector) and AddSource's forwardCPU
(deps/CustomOps/SourceOps/AddSource.cpp:33-89).  The elastic path has no
compiled reference; this checks the C oracle's step and loop, which every
elastic GPU parity test relies on, against a restatement that shares no code
with it.  Test infrastructure only."""
import numpy as np

from conftest import golden


def _step(st, lam, mu, rho, ax, bx, ay, by, dt, dx, dy, NX, NY, src=None):
    """One one_step on (13, NX+2, NY+2) fields (vx, vy, sxx, syy, sxy, mem1..8);
    ax, bx: (2, NX) with row 0 the integer grid (Julia row 1) and row 1 the
    half grid (Julia row 2); ay, by: (2, NY) likewise."""
    vx, vy, sxx, syy, sxy = (st[k].copy() for k in range(5))
    mem = [st[5 + k].copy() for k in range(8)]
    L, M, R = lam, mu, rho

    def box(i0, i1, j0, j1):  # 1-based inclusive Julia ranges -> numpy slices
        return slice(i0 - 1, i1), slice(j0 - 1, j1)

    def put(m, b, v):  # makevector: the new memory variable is zero off the box
        out = np.zeros_like(m)
        out[b] = v
        return out

    # fw1 (src/Core.jl:96-126): box rows 2:NX, columns 3:NY+1
    ij, i1j, i2j, i_1j = (box(2, NX, 3, NY + 1), box(3, NX + 1, 3, NY + 1),
                          box(4, NX + 2, 3, NY + 1), box(1, NX - 1, 3, NY + 1))
    ij_2, ij_1, ij1 = box(2, NX, 1, NY - 1), box(2, NX, 2, NY), box(2, NX, 4, NY + 2)
    lam_ = 0.5 * (L[i1j] + L[ij])
    mu_ = 0.5 * (M[i1j] + M[ij])
    lm = lam_ + 2 * mu_
    dvx = (27 * vx[i1j] - 27 * vx[ij] - vx[i2j] + vx[i_1j]) / (24 * dx)
    dvy = (27 * vy[ij] - 27 * vy[ij_1] - vy[ij1] + vy[ij_2]) / (24 * dy)
    rx = bx[1, 0:NX - 1][:, None], ax[1, 0:NX - 1][:, None]   # bx[2, 1:end-1]
    ry = by[0, 1:NY][None, :], ay[0, 1:NY][None, :]           # by[1, 2:end]
    mem[0] = put(mem[0], ij, rx[0] * mem[0][ij] + rx[1] * dvx)
    mem[1] = put(mem[1], ij, ry[0] * mem[1][ij] + ry[1] * dvy)
    dvx = dvx + mem[0][ij]
    dvy = dvy + mem[1][ij]
    sxx[ij] = sxx[ij] + (lm * dvx + lam_ * dvy) * dt
    syy[ij] = syy[ij] + (lm * dvy + lam_ * dvx) * dt

    # fw2 (src/Core.jl:128-155): box rows 3:NX+1, columns 2:NY
    ij, i_1j, i1j, i_2j = (box(3, NX + 1, 2, NY), box(2, NX, 2, NY), box(4, NX + 2, 2, NY),
                           box(1, NX - 1, 2, NY))
    ij_1, ij1, ij2 = box(3, NX + 1, 1, NY - 1), box(3, NX + 1, 3, NY + 1), box(3, NX + 1, 4, NY + 2)
    mu_ = 0.5 * (M[ij] + M[ij1])
    dvydx = (27 * vy[ij] - 27 * vy[i_1j] - vy[i1j] + vy[i_2j]) / (24 * dx)
    dvxdy = (27 * vx[ij1] - 27 * vx[ij] - vx[ij2] + vx[ij_1]) / (24 * dy)
    rx = bx[0, 1:NX][:, None], ax[0, 1:NX][:, None]           # bx[1, 2:end]
    ry = by[1, 0:NY - 1][None, :], ay[1, 0:NY - 1][None, :]   # by[2, 1:end-1]
    mem[2] = put(mem[2], ij, rx[0] * mem[2][ij] + rx[1] * dvydx)
    mem[3] = put(mem[3], ij, ry[0] * mem[3][ij] + ry[1] * dvxdy)
    dvydx = dvydx + mem[2][ij]
    dvxdy = dvxdy + mem[3][ij]
    sxy[ij] = sxy[ij] + mu_ * (dvydx + dvxdy) * dt

    # fw3 (src/Core.jl:158-184): box rows 3:NX+1, columns 3:NY+1
    ij, i_1j, i1j, i_2j = (box(3, NX + 1, 3, NY + 1), box(2, NX, 3, NY + 1),
                           box(4, NX + 2, 3, NY + 1), box(1, NX - 1, 3, NY + 1))
    ij_2, ij_1, ij1 = (box(3, NX + 1, 1, NY - 1), box(3, NX + 1, 2, NY),
                       box(3, NX + 1, 4, NY + 2))
    dsxx = (27 * sxx[ij] - 27 * sxx[i_1j] - sxx[i1j] + sxx[i_2j]) / (24 * dx)
    dsxy = (27 * sxy[ij] - 27 * sxy[ij_1] - sxy[ij1] + sxy[ij_2]) / (24 * dy)
    rx = bx[0, 1:NX][:, None], ax[0, 1:NX][:, None]           # bx[1, 2:end]
    ry = by[0, 1:NY][None, :], ay[0, 1:NY][None, :]           # by[1, 2:end]
    mem[4] = put(mem[4], ij, rx[0] * mem[4][ij] + rx[1] * dsxx)
    mem[5] = put(mem[5], ij, ry[0] * mem[5][ij] + ry[1] * dsxy)
    dsxx = dsxx + mem[4][ij]
    dsxy = dsxy + mem[5][ij]
    vx[ij] = vx[ij] + (dsxx + dsxy) * dt / R[ij]

    # fw4 (src/Core.jl:186-213): box rows 2:NX, columns 2:NY
    ij, i1j, i2j, i_1j = (box(2, NX, 2, NY), box(3, NX + 1, 2, NY), box(4, NX + 2, 2, NY),
                          box(1, NX - 1, 2, NY))
    i1j1, ij_1 = box(3, NX + 1, 3, NY + 1), box(2, NX, 1, NY - 1)
    ij1, ij2 = box(2, NX, 3, NY + 1), box(2, NX, 4, NY + 2)
    rho_ = 0.25 * (R[ij] + R[i1j] + R[i1j1] + R[ij1])
    dsxydx = (27 * sxy[i1j] - 27 * sxy[ij] - sxy[i2j] + sxy[i_1j]) / (24 * dx)
    dsyydy = (27 * syy[ij1] - 27 * syy[ij] - syy[ij2] + syy[ij_1]) / (24 * dy)
    rx = bx[1, 0:NX - 1][:, None], ax[1, 0:NX - 1][:, None]   # bx[2, 1:end-1]
    ry = by[1, 0:NY - 1][None, :], ay[1, 0:NY - 1][None, :]   # by[2, 1:end-1]
    mem[6] = put(mem[6], ij, rx[0] * mem[6][ij] + rx[1] * dsxydx)
    mem[7] = put(mem[7], ij, ry[0] * mem[7][ij] + ry[1] * dsyydy)
    dsxydx = dsxydx + mem[6][ij]
    dsyydy = dsyydy + mem[7][ij]
    vy[ij] = vy[ij] + (dsxydx + dsyydy) * dt / rho_

    # AddSource (AddSource.cpp:33-89): types 0 vx, 1 vy, 2 sxx, 3 syy, 4 sxy
    fields = {0: vx, 1: vy, 2: sxx, 3: syy, 4: sxy}
    if src is not None:
        for i, j, t, v in zip(*src):
            if int(t) in fields:
                fields[int(t)][i - 1, j - 1] += v
    return np.stack([vx, vy, sxx, syy, sxy] + mem)


def _case(seed):
    g = golden("elastic_small.npz")
    NX, NY = int(g["NX"]), int(g["NY"])
    shape = (NX + 2, NY + 2)
    prof = [g[k].reshape(2, -1) for k in ("ax", "bx", "ay", "by")]
    mat = [g[k].reshape(shape) for k in ("lam", "mu", "rho")]
    k = dict(dt=float(g["dt"]), dx=float(g["dx"]), dy=float(g["dy"]), NX=NX, NY=NY)
    return g, NX, NY, shape, prof, mat, k, np.random.default_rng(seed)


def test_step_matches_the_oracle(orc):
    """Random state (memory variables everywhere, so the zeroing off each box
    is exercised), sources of every type including the padded frame and an
    ignored type: the C oracle's step against this restatement."""
    g, NX, NY, shape, (ax, bx, ay, by), (lam, mu, rho), k, rng = _case(1)
    st = rng.standard_normal((13,) + shape)
    src = (np.array([15, 1, 4, 9, 12, 20]), np.array([10, 3, 24, 9, 7, 5]),
           np.array([2, 0, 4, 3, 1, 9]), rng.standard_normal(6))
    want = _step(st, lam, mu, rho, ax, bx, ay, by, src=src, **k)
    got = orc.elastic_step_fwd(st.reshape(-1), lam.reshape(-1), mu.reshape(-1),
                               rho.reshape(-1), ax.reshape(-1), bx.reshape(-1), ay.reshape(-1),
                               by.reshape(-1), k["dt"], k["dx"], k["dy"], NX, NY, *src)
    got = np.asarray(got).reshape(want.shape)
    for f in range(13):  # the same operations in the same order: bit-identical
        assert np.array_equal(got[f], want[f]), f


def test_loop_matches_the_oracle_and_the_fixture(orc):
    """The loop of src/Core.jl:31-94 (slot 0 zero, slot n = one_step of slot
    n-1 with source row n-1) over the fixture's model and sources: the whole
    history against the oracle's, and the receiver traces against the
    committed fixture."""
    g, NX, NY, shape, (ax, bx, ay, by), (lam, mu, rho), k, _ = _case(2)
    T = int(g["NSTEP"])
    src = (g["srci"], g["srcj"], g["srctype"])
    st = np.zeros((13,) + shape)
    hist = [st]
    for n in range(1, T + 1):
        st = _step(st, lam, mu, rho, ax, bx, ay, by, src=src + (g["srcv"][n - 1],), **k)
        hist.append(st)
    hist = np.stack(hist)
    rcvv, ref = orc.elastic_forward(NX, NY, T, k["dt"], k["dx"], k["dy"], g["ax"], g["bx"],
                                    g["ay"], g["by"], g["lam"], g["mu"], g["rho"], *src,
                                    g["srcv"], g["rcvi"], g["rcvj"], g["rcvtype"],
                                    keep_history=True)
    for f in range(13):
        assert np.array_equal(ref[:, f], hist[:, f]), f
    tr = np.stack([hist[:, t, i - 1, j - 1] for i, j, t in
                   zip(g["rcvi"], g["rcvj"], g["rcvtype"])])
    assert np.linalg.norm(tr - g["rcvv"]) <= 1e-12 * np.linalg.norm(g["rcvv"])
