"""The reference's output step (xt_slab_dump, src/postprocess.f90:106-378):
record counts and formats of the dump files, the Gauss-point strain equal
to the strain rows applied to the dumped nodal displacement, the stress
equal to the elastic law applied to it (zero at failed points), and the
damage, stored energy and element status equal to the slab state."""
import numpy as np
import pytest

from conftest import rod_problem

pytestmark = pytest.mark.gpu

NSLAB = 4


def read_rows(path):
    return [line.split() for line in open(path) if line.strip()]


def test_dump_records_match_the_state(xt, tmp_path):
    pr = rod_problem(xt)
    cfg = xt.SlabConfig.make(amplitude=1000.0, nipc=32, n1=10, n2=2, im=30, precision=2,
                             tol=1e-8, Dc=0.02, overlap=1)
    s = xt.SlabSolver(pr, cfg)
    s.set_state(ws=np.full(s.ngp, 31.7))
    job = str(tmp_path / "rod")
    states = []
    for k in range(NSLAB):
        s.step()
        s.dump(job, truncate=(k == 0))
        states.append(s.state())
    nn, ne = pr.sizes()[:2]
    ngp = 8 * ne
    Nx, Ny, Nz = (a.reshape(ngp, 8) for a in pr.strain_rows())
    _, conn = pr.mesh()
    times = [float(r[0]) for r in read_rows(job + ".time")]
    assert len(times) == NSLAB and all(b > a for a, b in zip(times, times[1:]))
    disp = np.array(read_rows(job + ".disp"), float).reshape(NSLAB, nn, 3)
    strain = np.array(read_rows(job + "_0.strain"), float).reshape(NSLAB, ngp, 6)
    stress = np.array(read_rows(job + "_0.stress"), float).reshape(NSLAB, ngp, 6)
    damage = np.array(read_rows(job + "_0.damage"), float).reshape(NSLAB, ngp)
    energy = np.array(read_rows(job + "_0.energy"), float).reshape(NSLAB, ngp)
    status = np.array(read_rows(job + "_0.status"), int).reshape(NSLAB, ne)
    line = open(job + "_0.stress").readline()
    assert len(line.rstrip("\n")) == 6 * 18 and line[2:4] in ("0.", "-0")
    E, nu = 2.0e5, 0.3
    c = E / ((1 + nu) * (1 - 2 * nu))
    Dm = np.zeros((6, 6))
    Dm[:3, :3] = c * nu
    Dm[np.arange(3), np.arange(3)] = c * (1 - nu)
    Dm[np.arange(3, 6), np.arange(3, 6)] = c * (1 - 2 * nu) / 2
    for k in range(NSLAB):
        u = disp[k][conn[np.arange(ngp) // 8] - 1]  # ngp x 8 nodes x 3
        e = np.stack([(Nx * u[:, :, 0]).sum(1), (Ny * u[:, :, 1]).sum(1), (Nz * u[:, :, 2]).sum(1),
                      (Ny * u[:, :, 0] + Nx * u[:, :, 1]).sum(1),
                      (Nz * u[:, :, 1] + Ny * u[:, :, 2]).sum(1),
                      (Nz * u[:, :, 0] + Nx * u[:, :, 2]).sum(1)], 1)
        live = np.repeat(states[k]["elesta"], 8) == 1
        e[~live] = 0.0
        sg = e @ Dm.T
        scale_e, scale_s = np.abs(e).max(), np.abs(sg).max()
        assert np.max(np.abs(strain[k] - e)) <= 1e-6 * scale_e, k
        assert np.max(np.abs(stress[k] - sg)) <= 1e-6 * scale_s, k
        assert np.all(strain[k][~live] == 0.0) and np.all(stress[k][~live] == 0.0)
        assert np.allclose(damage[k], states[k]["D"], rtol=1e-15, atol=0)
        assert np.allclose(energy[k], states[k]["ws"], rtol=1e-15, atol=0)
        assert np.array_equal(status[k], states[k]["elesta"])
    assert (status[-1] == 0).any()  # elements failed during the run
    s.close()
    pr.close()
