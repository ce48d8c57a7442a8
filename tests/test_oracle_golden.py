"""Pin the CPU oracle to golden vectors captured from the reference itself.

Every fixture in ``tests/golden`` holds seeded inputs and the exact array that
the reference's ``verify_stencil`` compares against (``make_golden.py``).  The
oracle must reproduce those arrays bit for bit; for horizontal diffusion the
reference's numpy backend output must match as well.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import stencils as ora
from tests.conftest import golden_cases, load_golden

CASES = {k: v for k, v in golden_cases().items() if not k.startswith("_")}


def _bits_equal(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    assert a.shape == b.shape and a.dtype == b.dtype
    view = {8: np.uint64, 4: np.uint32, 2: np.uint16}[a.dtype.itemsize]
    return np.array_equal(a.view(view), b.view(view))


def _oracle_outputs(meta, data):
    domain, halo, kind = tuple(meta["domain"]), tuple(meta["halo"]), meta["kind"]
    fields = {n: data[f"in_{n}"] for n in meta["args"]}
    params = meta["params"]
    if kind == "hdiff":
        return {"out": ora.hdiff(fields["inp"], fields["coeff"], domain, halo)}
    if kind == "vadv":
        return ora.vadv(fields, domain, halo, params.get("all_components", False))
    if kind == "copy":
        return {"out": ora.copy(fields["inp"], domain, halo)}
    if kind == "laplacian":
        along = (params.get("along_x", True), params.get("along_y", True), params.get("along_z", False))
        return {"out": ora.laplacian(fields["inp"], domain, halo, along)}
    if kind == "onesided_average":
        return {"out": ora.onesided_average(fields["inp"], domain, halo, params["axis"])}
    if kind == "symmetric_average":
        return {"out": ora.symmetric_average(fields["inp"], domain, halo, params["axis"])}
    raise AssertionError(kind)


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_bitwise(name):
    meta = CASES[name]
    data = load_golden(name)
    got = _oracle_outputs(meta, data)
    for out in meta["outputs"]:
        assert _bits_equal(got[out], data[f"expected_{out}"]), f"{name}:{out}"


@pytest.mark.parametrize("name", sorted(k for k, v in CASES.items() if v["kind"] == "hdiff"))
def test_reference_numpy_backend_agrees(name):
    data = load_golden(name)
    assert _bits_equal(data["numpy_backend_out"], data["expected_out"])


def test_stream_scalars(golden):
    for key, (a, b, c) in golden["_stream_scalars"].items():
        dtype, ntimes = key.rsplit("_", 1)
        got = ora.stream_expected_scalars(int(ntimes), dtype)
        assert [float(x) for x in got] == [a, b, c]


def test_planted_mistake_is_caught():
    """A wrong limiter sign in a copy of the oracle must miss the golden."""
    data = load_golden("hdiff_f64_h2")
    meta = CASES["hdiff_f64_h2"]
    inp, coeff = data["in_inp"], data["in_coeff"]
    domain, halo = tuple(meta["domain"]), tuple(meta["halo"])
    # same formula, limiter condition flipped (< 0 instead of > 0)
    lap = np.zeros_like(inp)
    lap[1:-1, 1:-1] = 4 * inp[1:-1, 1:-1] - (
        inp[2:, 1:-1] + inp[:-2, 1:-1] + inp[1:-1, 2:] + inp[1:-1, :-2]
    )
    flx = np.zeros_like(inp)
    flx[:-1] = lap[1:] - lap[:-1]
    flx[:-1] = np.where(flx[:-1] * (inp[1:] - inp[:-1]) < 0, 0, flx[:-1])
    fly = np.zeros_like(inp)
    fly[:, :-1] = lap[:, 1:] - lap[:, :-1]
    fly[:, :-1] = np.where(fly[:, :-1] * (inp[:, 1:] - inp[:, :-1]) < 0, 0, fly[:, :-1])
    res = np.zeros_like(inp)
    res[1:-1, 1:-1] = inp[1:-1, 1:-1] - coeff[1:-1, 1:-1] * (
        flx[1:-1, 1:-1] - flx[:-2, 1:-1] + fly[1:-1, 1:-1] - fly[1:-1, :-2]
    )
    wrong = res[ora.inner_slice(domain, halo)]
    assert not _bits_equal(wrong, data["expected_out"])


def test_bf16_rounding_known_values():
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e38, 1e-40, 0.0, -0.0], dtype=np.float32)
    bits = ora.f32_to_bf16_bits(x)
    back = ora.bf16_bits_to_f32(bits)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: rounds to even (1.0)
    assert back[0] == 1.0 and back[1] == 1.0
    # 1 + 3*2^-9 rounds up to 1 + 2^-7
    assert back[2] == np.float32(1.0078125)
    assert back[3] == -2.5
    assert np.signbit(back[7]) and back[6] == 0
    nan = ora.bf16_bits_to_f32(ora.f32_to_bf16_bits(np.array([np.nan], np.float32)))
    assert np.isnan(nan[0])
