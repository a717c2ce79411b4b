"""Request farm (bemgpu_farm_*): several lanes solving at once must give the
same spectral powers as one CalcHeatTransfer call after another, bit for bit
(every kernel of the solve is deterministic), keep the reference's error
behaviour per request, and drop queued requests on cancel / destroy.
The reference's counterpart is the MPI task farm, src/transfer-mpi.cpp:25-190."""
import numpy as np
import pytest

from bem_gb300 import _lib, api, mesh

pytestmark = pytest.mark.gpu


def _systems(level=1, gaps=(0.05, 0.2)):
    v, t = mesh.icosphere(1.0, level, jitter=0.02, seed=12345)
    b2 = mesh.Body.from_mesh(v, t)
    d = api.FixedLorentz(*api.SIC_CONFIG)
    return [api.parseShapes(b2.translated(mesh.gap_translation(v, v, g)), b2, d, d) for g in gaps]


@pytest.mark.parametrize("precision", [_lib.PREC_FP64, _lib.PREC_MIXED_LA])
@pytest.mark.parametrize("lanes", [1, 3])
def test_farm_matches_serial_solves(precision, lanes):
    systems = _systems()
    jobs = [(1e-6, f, 300.0, 0.0, *systems[i % 2]) for i, f in enumerate(np.linspace(0.085, 0.125, 7))]
    serial = [api.CalcHeatTransfer(*j, precision=precision, strict=False) for j in jobs]
    with api.Farm(lanes) as farm:
        infos = []
        got = farm.map(jobs, precision=precision, strict=False, infos=infos)
    assert got == serial
    assert all(i["ms_fill"] > 0 for i in infos)


def test_farm_out_of_order_collection_and_cancel():
    systems = _systems(level=2, gaps=(0.1,))
    top, s, t = systems[0]
    with api.Farm(2) as farm:
        tickets = [farm.submit(1e-6, f, 300.0, 0.0, top, s, t, precision=_lib.PREC_MIXED_LA)
                   for f in np.linspace(0.09, 0.12, 6)]
        # the last request is queued behind five others on two lanes
        cancelled = farm.cancel(tickets[-1])
        Ps = [farm.result(tk, strict=False) for tk in reversed(tickets[:-1])]
        assert all(np.isfinite(Ps)) and all(P > 0 for P in Ps)
        if cancelled:
            with pytest.raises(_lib.BemGpuError) as e:
                farm.result(tickets[-1])
            assert e.value.code == _lib.ERR_CANCELLED
        else:
            assert farm.result(tickets[-1], strict=False) > 0
        # a collected ticket is gone
        with pytest.raises(_lib.BemGpuError) as e:
            farm.poll(tickets[0])
        assert e.value.code == _lib.ERR_ARG


def test_farm_rejects_bad_requests():
    systems = _systems(level=1, gaps=(0.1,))
    top, s, t = systems[0]
    with api.Farm(1) as farm:
        with pytest.raises(_lib.BemGpuError) as e:
            farm.submit(1e-6, 0.1, 300.0, 0.0, top, t, s, precision=7)
        assert e.value.code == _lib.ERR_ARG
        with pytest.raises(_lib.BemGpuError):
            farm.submit(1e-6, 0.1, 300.0, 0.0, s, s, t)  # size(top) != size(s) + size(t)
        # the farm still serves after rejected requests
        assert farm.result(farm.submit(1e-6, 0.1, 300.0, 0.0, top, s, t)) == \
            api.CalcHeatTransfer(1e-6, 0.1, 300.0, 0.0, top, s, t)


def test_farm_destroy_drops_queued_requests():
    systems = _systems(level=2, gaps=(0.1,))
    farm = api.Farm(1)
    for f in np.linspace(0.09, 0.12, 4):
        farm.submit(1e-6, f, 300.0, 0.0, *systems[0], precision=_lib.PREC_MIXED_LA)
    farm.close()  # returns after the running request; the queued ones are dropped
    assert farm.handle is None


def _system_level(level, gap):
    v, t = mesh.icosphere(1.0, level, jitter=0.02, seed=12345)
    b2 = mesh.Body.from_mesh(v, t)
    d = api.FixedLorentz(*api.SIC_CONFIG)
    return api.parseShapes(b2.translated(mesh.gap_translation(v, v, gap)), b2, d, d)


def test_uneven_sizes_same_alone_and_in_the_mix():
    """Requests of different N (icospheres L1 and L2, two gaps) interleaved on
    three lanes give exactly the spectral power each gives alone."""
    systems = [_system_level(1, 0.05), _system_level(2, 0.1), _system_level(1, 0.3), _system_level(2, 0.02)]
    jobs = [(1e-6, f, 300.0, 0.0, *systems[i % 4]) for i, f in enumerate(np.linspace(0.085, 0.125, 8))]
    alone = [api.CalcHeatTransfer(*j, precision=_lib.PREC_MIXED_LA, strict=False) for j in jobs]
    with api.Farm(3) as farm:
        infos = []
        mixed = farm.map(jobs, precision=_lib.PREC_MIXED_LA, strict=False, infos=infos)
    assert mixed == alone
    assert all(i["ms_latency"] >= i["ms_queued"] >= 0 for i in infos)


def test_footprint_bounds_the_workspace():
    """bemgpu_solve_footprint is the admission figure: it must cover what a
    solve allocates, without overstating it by much."""
    L = _lib.load()
    for level, prec, solver in ((1, _lib.PREC_FP64, 0), (2, _lib.PREC_FP64, 0), (2, _lib.PREC_MIXED_LA, 0),
                                (2, _lib.PREC_MIXED_LA, 2)):
        ctx = api.Context(0)
        ctx.set_solver(solver)
        top2, s2, t2 = api.parseShapes(*_bodies(level, 0.1), api.FixedLorentz(*api.SIC_CONFIG),
                                       api.FixedLorentz(*api.SIC_CONFIG), ctx)
        api.CalcHeatTransfer(1e-6, 0.1, 300.0, 0.0, top2, s2, t2, precision=prec, strict=False)
        held = L.bemgpu_ctx_workspace_bytes(ctx.handle)
        fp = api.solve_footprint(s2, t2, prec, ctx)
        # the escalating mode also counts what an escalation would add (a copy
        # of W, the FP64-class LU's blocks, the FP64 fallback's buffers), which
        # a well-conditioned solve never allocates
        n, ns2 = 2 * (s2.rwgs + t2.rwgs), 2 * s2.rwgs
        nt2 = n - ns2
        unused = 0
        if prec != _lib.PREC_FP64 and solver == 0:
            unused = 16 * n * n + 16 * n * nt2 + 32 * ns2 * nt2 + 32 * n * 512 + 2 * 5 * 2 * (2 * n + 128) * 1024
        assert held <= fp <= 1.5 * held + unused + (64 << 20), (level, prec, solver, held, fp)
        if solver == 2:
            # FP64-class only: no complex64 factors
            assert fp < api.solve_footprint(s2, t2, prec)
        assert L.bemgpu_ctx_trim(ctx.handle) == 0 and L.bemgpu_ctx_workspace_bytes(ctx.handle) == 0
        # a trimmed context solves again and gives the same answer
        P1 = api.CalcHeatTransfer(1e-6, 0.1, 300.0, 0.0, top2, s2, t2, precision=prec, strict=False)
        L.bemgpu_ctx_trim(ctx.handle)
        P2 = api.CalcHeatTransfer(1e-6, 0.1, 300.0, 0.0, top2, s2, t2, precision=prec, strict=False)
        assert P1 == P2
        del top2, s2, t2
        ctx.close()


def _bodies(level, gap):
    v, t = mesh.icosphere(1.0, level, jitter=0.02, seed=12345)
    b2 = mesh.Body.from_mesh(v, t)
    return b2.translated(mesh.gap_translation(v, v, gap)), b2


def test_admission_by_footprint():
    """A budget that holds one solve at a time serialises the lanes (same
    results); a request larger than the budget fails with BEMGPU_ERR_OOM."""
    small = _system_level(1, 0.1)
    big = _system_level(2, 0.1)
    fp_big = api.solve_footprint(big[1], big[2], _lib.PREC_MIXED_LA)
    fp_small = api.solve_footprint(small[1], small[2], _lib.PREC_MIXED_LA)
    jobs = [(1e-6, f, 300.0, 0.0, *(big if i % 2 else small)) for i, f in enumerate(np.linspace(0.09, 0.12, 6))]
    alone = [api.CalcHeatTransfer(*j, precision=_lib.PREC_MIXED_LA, strict=False) for j in jobs]
    with api.Farm(3) as farm:
        farm.budget = fp_big + fp_small // 2   # room for one large solve and half a small one
        assert farm.budget == fp_big + fp_small // 2
        got = farm.map(jobs, precision=_lib.PREC_MIXED_LA, strict=False)
        assert got == alone
        farm.budget = fp_big // 2
        tk = farm.submit(*jobs[1], precision=_lib.PREC_MIXED_LA)
        with pytest.raises(_lib.BemGpuError) as e:
            farm.result(tk)
        assert e.value.code == _lib.ERR_OOM
        farm.budget = 4 * fp_big
        assert farm.result(farm.submit(*jobs[1], precision=_lib.PREC_MIXED_LA), strict=False) == alone[1]
