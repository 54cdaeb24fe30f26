"""The device task-list builder of one- and two-site pivots (builder.cu;
precalc_blockStructure, tensors/DmrgIndexGymnastics.h:487-590 and :699-856): on a
device context an abelian pivot matches its chains on the GPU; with
VMPS_HOST_BUILDER=1 the host builder makes them.  Both give the same chain list in the
same order (block indices and coefficients bit for bit) and the same reference task
count, so the plans and the HxV bits agree too: Hubbard U(1)xU(1) pivots of the C2
chain (two-site and one-site), Heisenberg U(1) pivots, and a union pivot (three
quantum-number components, two sectors) of the C5 spectral workload."""
import numpy as np
import pytest

from vmps_gb300 import models
from vmps_gb300.pivot import PivotMatrix1, PivotMatrix2
from vmps_gb300.workloads import heisenberg_two_site, hubbard_two_site

pytestmark = pytest.mark.gpu


def _both(monkeypatch, make):
    monkeypatch.setenv("VMPS_HOST_BUILDER", "1")
    Hh = make()
    monkeypatch.delenv("VMPS_HOST_BUILDER")
    Hd = make()
    return Hh, Hd


def _same(Hh, Hd, v=None):
    ih, ch, th = Hh.chains()
    idv, cd, td = Hd.chains()
    assert len(ih) > 0
    assert np.array_equal(ih, idv)
    assert np.array_equal(ch.view(np.int64), cd.view(np.int64))
    assert th == td
    if v is not None:
        for prec in ("fp64", "bf16x3"):
            assert np.array_equal(Hh.apply(v, prec), Hd.apply(v, prec)), prec


@pytest.mark.parametrize("D", [256, 2048])
def test_device_builder_equals_host_builder_hubbard(gpu_ctx, monkeypatch, D):
    model, mps, Lenv, Renv, W1, W2, V, info = hubbard_two_site(gpu_ctx, L=32, D=D, seed=4)
    Hh, Hd = _both(monkeypatch, lambda: PivotMatrix2(gpu_ctx, model.sym, Lenv, Renv, W1, W2, V))
    _same(Hh, Hd, np.random.default_rng(1).standard_normal(Hh.dim))
    Hh.close()
    Hd.close()


def test_device_builder_equals_host_builder_heisenberg(gpu_ctx, monkeypatch):
    model, mps, Lenv, Renv, W1, W2, V, info = heisenberg_two_site(gpu_ctx, L=24, D=64, seed=2)
    Hh, Hd = _both(monkeypatch, lambda: PivotMatrix2(gpu_ctx, model.sym, Lenv, Renv, W1, W2, V))
    _same(Hh, Hd, np.random.default_rng(2).standard_normal(Hh.dim))
    Hh.close()
    Hd.close()


def test_device_builder_equals_host_builder_union(gpu_ctx, monkeypatch):
    """two spin sectors of c_k|0> as one union pivot (a part tag as third component)"""
    from vmps_gb300.dmrg import dmrg2
    from vmps_gb300.mps import RandomMPS
    from vmps_gb300.spectral import SpectralPivot
    from vmps_gb300.union import UnionPivot2
    L, l = 12, 5
    model = models.hubbard_u1xu1(L, t=1.0, U=4.0)
    mps = RandomMPS(model, (L, 0), 48, seed=3).canonicalize(0, 0)
    dmrg2(gpu_ctx, model, mps, n_sweeps=1, Dmax=48, precision="fp64")
    mps.canonicalize(l, l + 1)
    sp = SpectralPivot(gpu_ctx, model, mps, l)
    parts = [sp.sector(s) for s in ("up", "dn")]
    Hh, Hd = _both(monkeypatch, lambda: UnionPivot2(gpu_ctx, model.sym, model.W[l], model.W[l + 1], parts))
    _same(Hh.H, Hd.H, np.random.default_rng(3).standard_normal(Hh.H.dim))
    Hh.close()
    Hd.close()


@pytest.mark.parametrize("case", ["hubbard", "heis"])
def test_device_builder_equals_host_builder_one_site(gpu_ctx, monkeypatch, case):
    from helpers import pivot1_case
    if case == "hubbard":
        model, mps, Lenv, Renv, W, V = pivot1_case("hubb", L=24, D=512, site=11, seed=5, profile="gaussian")
    else:
        model, mps, Lenv, Renv, W, V = pivot1_case("heis", L=24, D=256, site=11, seed=6, profile="gaussian")
    Hh, Hd = _both(monkeypatch, lambda: PivotMatrix1(gpu_ctx, model.sym, Lenv, Renv, W, V))
    _same(Hh, Hd, np.random.default_rng(4).standard_normal(Hh.dim))
    Hh.close()
    Hd.close()
