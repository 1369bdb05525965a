"""The allocation-free damage entry point, xt_damage_device, against the
allocating one, xt_damage.

xt_damage_device takes device pointers and keeps its scratch in a static
array of the library's device image, so this file runs last (its name sorts
after the other test files): the static scratch then has been untouched by
the other tests, or reused after them, and both orders must pass.  Device
buffers for the test come from torch (test plumbing only; the entry point
itself allocates nothing).
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rod_problem

KEYS = ["eps_old", "eps_pl", "sig_eff", "sig_back", "p", "D", "ws", "del_po", "sig_d"]
XT_ERR_ARG = -10
MAX_NIP = 65536


def damage_case(xt, nip=512):
    """4x4x12 rod, a seeded random displacement field of plastic size, stored
    energy seeded just below the damage threshold so damage grows."""
    pr = rod_problem(xt)
    xyz, conn = pr.mesh()
    nn, ne = len(xyz), len(conn)
    Nx, Ny, Nz = pr.strain_rows()
    nodes = np.repeat(conn, 8, axis=0).ravel().astype(np.int32)
    Nt = xt.nt_table(nip, np.array([0.0, 0.25, 0.5]), 2 * np.pi * 20)
    sol = np.random.default_rng(7).standard_normal(6 * 3 * nn) * 4e-4
    ngp = 8 * ne
    st = {k: np.zeros(ngp * 6) for k in KEYS[:4]}
    st.update({k: np.zeros(ngp) for k in KEYS[4:]})
    st["ws"][:] = 31.7
    pr.close()
    return dict(ne=ne, nn=nn, nip=nip, nodes=nodes, Nx=Nx, Ny=Ny, Nz=Nz, Nt=Nt, sol=sol,
                ym=np.full(ngp, 2.0e5), nu=np.full(ngp, 0.3), state=st)


@pytest.mark.gpu
def test_device_entry_matches_xt_damage_over_two_calls(xt):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    xt.lib().xt_init(0)
    d = damage_case(xt)
    ref = {k: v.copy() for k, v in d["state"].items()}
    dev = {k: torch.from_numpy(v.copy()).cuda() for k, v in d["state"].items()}
    inp = {k: torch.from_numpy(np.ascontiguousarray(d[k])).cuda()
           for k in ["nodes", "Nx", "Ny", "Nz", "Nt", "sol", "ym", "nu"]}
    torch.cuda.synchronize()
    ptr = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    plastic_total = 0
    for call in range(2):
        xt.damage(d["ne"], d["nn"], d["nip"], d["nodes"], d["Nx"], d["Ny"], d["Nz"], d["Nt"],
                  d["sol"], d["ym"], d["nu"], ref)
        counts = (C.c_ulonglong * 3)()
        st = xt.lib().xt_damage_device(
            d["ne"], d["nn"], 3, 8, 3, 8, 6, d["nip"],
            *[ptr(inp[k]) for k in ["nodes", "Nx", "Ny", "Nz", "Nt", "sol", "ym", "nu"]],
            *[ptr(dev[k]) for k in KEYS], counts)
        assert st == 0, xt.lib().xt_last_error()
        torch.cuda.synchronize()
        for k in KEYS:
            got = dev[k].cpu().numpy()
            assert np.array_equal(got, ref[k]), (call, k)
        ngp = 8 * d["ne"]
        # every (point, step) is counted once as screened-elastic or exact
        assert counts[1] + counts[2] == ngp * d["nip"]
        plastic_total += counts[0]
    assert plastic_total > 0 and ref["D"].max() > 0.0  # the case exercises the plastic path


def test_device_entry_rejects_oversize_nip(xt):
    """nip above the static scratch is refused on the host with a message,
    before any device work (runs without a GPU)."""
    one_i = np.zeros(1, np.int32)
    one_d = np.zeros(1)
    p_i = C.c_void_p(one_i.ctypes.data)
    p_d = C.c_void_p(one_d.ctypes.data)
    st = xt.lib().xt_damage_device(1, 1, 3, 8, 3, 8, 6, MAX_NIP + 1, p_i, *([p_d] * 16), None)
    assert st == XT_ERR_ARG
    msg = xt.lib().xt_last_error().decode()
    assert "exceeds the static scratch" in msg and str(MAX_NIP) in msg
    xt.lib().xt_clear_error()


@pytest.mark.gpu
def test_device_entry_waits_for_writes_on_callers_stream(xt):
    """The caller's kernels write the state on a stream of its own and the
    call follows without a host synchronisation: the entry point waits for
    that work (device-wide) before it reads, so the result equals
    xt_damage's on the written values."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    xt.lib().xt_init(0)
    d = damage_case(xt)
    ref = {k: v.copy() for k, v in d["state"].items()}
    src = {k: torch.from_numpy(v.copy()).cuda() for k, v in d["state"].items()}
    dev = {k: torch.full_like(v, float("nan")) for k, v in src.items()}
    inp = {k: torch.from_numpy(np.ascontiguousarray(d[k])).cuda()
           for k in ["nodes", "Nx", "Ny", "Nz", "Nt", "sol", "ym", "nu"]}
    xt.damage(d["ne"], d["nn"], d["nip"], d["nodes"], d["Nx"], d["Ny"], d["Nz"], d["Nt"],
              d["sol"], d["ym"], d["nu"], ref)
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        # keep the stream busy for a while, then write the real state
        if hasattr(torch.cuda, "_sleep"):
            torch.cuda._sleep(200_000_000)
        else:
            m = torch.randn(2048, 2048, device="cuda")
            for _ in range(50):
                m = torch.tanh(m @ m)
        for k in KEYS:
            dev[k].copy_(src[k])
    ptr = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    st = xt.lib().xt_damage_device(
        d["ne"], d["nn"], 3, 8, 3, 8, 6, d["nip"],
        *[ptr(inp[k]) for k in ["nodes", "Nx", "Ny", "Nz", "Nt", "sol", "ym", "nu"]],
        *[ptr(dev[k]) for k in KEYS], None)
    assert st == 0, xt.lib().xt_last_error()
    torch.cuda.synchronize()
    for k in KEYS:
        assert np.array_equal(dev[k].cpu().numpy(), ref[k]), k
