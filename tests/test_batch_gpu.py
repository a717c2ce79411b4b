"""The batched small-solve path (bemgpu_heat_transfer_batch): several
CalcHeatTransfer requests (src/HeatTransfer.cpp:8-59) with their fills in one
launch pair and, for equal sizes, their complex64 LU panels in one cooperative
launch per block column.  Every result must equal the one-at-a-time solve's
bit for bit: a frequency sweep of one geometry, requests of different
geometries and sizes, both precisions."""
import numpy as np
import pytest

import bench
from bem_gb300 import api, mesh, _lib

pytestmark = pytest.mark.gpu


def _cube_pair(nsub, gap, ctx):
    v, t = mesh.cube(1.0, nsub)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated(mesh.gap_translation(v, v, gap))
    d = api.FixedLorentz(*api.SIC_CONFIG)
    return api.parseShapes(b1, b2, d, d, ctx)


@pytest.mark.parametrize("precision", [_lib.PREC_MIXED_LA, _lib.PREC_FP64])
def test_sweep_batch_equals_single_solves(precision):
    ctx = api.Context(0)
    top, s, t = _cube_pair(3, 0.1, ctx)
    freqs = [0.085, 0.0983, 0.11, 0.116, 0.125] if precision != _lib.PREC_FP64 else [0.09, 0.116]
    jobs = [(1e-6, f, 300.0, 0.0, top, s, t) for f in freqs]
    single = [api.CalcHeatTransfer(*j, precision=precision) for j in jobs]
    infos = []
    batch = api.CalcHeatTransferBatch(jobs, precision=precision, infos=infos)
    assert batch == single
    assert all(i["pairs_near"] > 0 for i in infos)


def test_mixed_geometries_and_sizes_in_one_batch():
    ctx = api.Context(0)
    reqs = bench.tip_requests(bench.WORKLOADS["tip"])[:3]
    sic = api.FixedLorentz(*bench.SIC)
    jobs = []
    for (b1, b2, eV) in reqs:
        top, s, t = api.parseShapes(b1, b2, sic, sic, ctx)
        jobs.append((1e-6, eV, 300.0, 0.0, top, s, t))
    jobs.append((1e-6, 0.1, 300.0, 0.0, *_cube_pair(2, 0.05, ctx)))
    single = [api.CalcHeatTransfer(*j, precision=_lib.PREC_MIXED_LA, strict=False) for j in jobs]
    batch = api.CalcHeatTransferBatch(jobs, precision=_lib.PREC_MIXED_LA, strict=False)
    assert batch == single


def test_batch_footprint_and_limits():
    L = _lib.load()
    one = L.bemgpu_batch_footprint(1, 288, 288, _lib.PREC_MIXED_LA)
    four = L.bemgpu_batch_footprint(4, 288, 288, _lib.PREC_MIXED_LA)
    assert 0 < one < four < 4 * one + L.bemgpu_solve_footprint(288, 288, _lib.PREC_MIXED_LA)
    ctx = api.Context(0)
    top, s, t = _cube_pair(1, 0.1, ctx)
    with pytest.raises(_lib.BemGpuError):
        api.CalcHeatTransferBatch([(1e-6, 0.1, 300.0, 0.0, top, s, t)] * 65)


def test_farm_batches_queued_requests_with_the_same_results():
    """Continuous batching in the request farm: with a batch size of 4, lanes
    take queued requests of equal sizes together; every result equals the
    unbatched farm's and the single solve's."""
    ctx = api.Context(0)
    top, s, t = _cube_pair(3, 0.1, ctx)
    jobs = [(1e-6, f, 300.0, 0.0, top, s, t) for f in np.linspace(0.08, 0.13, 9)]
    single = [api.CalcHeatTransfer(*j, precision=_lib.PREC_MIXED_LA) for j in jobs]
    with api.Farm(2, 0, batch=4) as farm:
        batched = farm.map(jobs, precision=_lib.PREC_MIXED_LA)
    assert batched == single
