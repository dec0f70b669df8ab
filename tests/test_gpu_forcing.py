"""Forcing regions (src/forcing.jl): point forcing against the oracle's
regularization with unit weights, line and area forcing against the
operators they are built from, and the accumulation of several regions."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import ilm_oracle as O


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max()


def _setup():
    import immersedlayers as il
    from immersedlayers import bodies as B
    h = 0.04
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), h)
    og = O.Grid.physical((-2.0, 2.0), (-2.0, 2.0), h)
    base = il.SurfaceScalarCache(B.circle(0.5, ds=1.4 * h), g)
    return il, B, h, g, og, base


def test_point_forcing_matches_oracle(cuda):
    il, B, h, g, og, base = _setup()
    px = np.array([0.3, -0.71, 1.05])
    py = np.array([0.2, 0.44, -0.9])
    strength = np.array([1.0, -2.5, 0.75])

    def fcn(s, y, t, fcache, pp):
        import torch
        s.data.copy_(torch.tensor(strength * (1.0 + t), device="cuda"))

    fr = il.forcing_regions(il.PointForcingModel((px, py), fcn), base)
    out = il.zeros_grid(base)
    il.apply_forcing_(out, None, None, 0.5, fr)
    oc = O.SurfaceCache(px, py, np.ones(3), np.zeros(3), np.ones(3), og)
    ref = O.regularize_scalar(oc, strength * 1.5)
    assert rel(out.numpy_components(), ref) < 1e-12


def test_line_area_forcing_and_accumulation(cuda):
    import torch
    il, B, h, g, og, base = _setup()
    line = B.circle(0.8, ds=1.4 * h, center=(0.2, -0.1))
    area = B.ellipse(0.6, 0.3, ds=1.4 * h, center=(-0.4, 0.5))

    def line_fcn(s, y, t, fcache, pp):
        s.data.fill_(pp["q"])

    field = il.zeros_grid(base)
    field.data.normal_()

    def area_fcn(s, y, t, fcache, pp):
        s.data.copy_(field.data)

    models = [il.LineForcingModel(line, line_fcn), il.AreaForcingModel(area, area_fcn),
              il.AreaForcingModel(lambda s, y, t, fc, pp: s.data.fill_(0.25))]
    fr = il.forcing_regions(models, base)
    out = il.zeros_grid(base)
    out.data.fill_(7.0)  # cleared by apply_forcing!
    il.apply_forcing_(out, None, None, 0.0, fr, phys_params={"q": 2.0})
    lc = il.SurfaceScalarCache(line, g)
    q = il.ScalarData(torch.full((len(line),), 2.0, dtype=torch.float64, device="cuda"))
    r_line = il.regularize_(il.zeros_grid(lc), q, lc).data
    m = il.mask(il.SurfaceScalarCache(area, g)).data
    expect = r_line + field.data * m + 0.25
    torch.cuda.synchronize()
    assert float((out.data - expect).abs().max() / expect.abs().max()) < 1e-13
    # the line region alone, twice: the accumulating scatter adds
    fr1 = il.forcing_regions([il.LineForcingModel(line, line_fcn), il.LineForcingModel(line, line_fcn)], base)
    il.apply_forcing_(out, None, None, 0.0, fr1, phys_params={"q": 2.0})
    assert float((out.data - 2 * r_line).abs().max() / r_line.abs().max()) < 1e-13
