"""The committed golden vectors (tests/golden/oracle_golden.npz, made by
tests/golden/make_golden.py from the CPU oracle): the oracle must reproduce them bit for
bit (CPU), and the CUDA library must match them under the parity bars (GPU)."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden  # noqa: E402

GOLDEN = os.path.join(HERE, "golden", "oracle_golden.npz")


@pytest.fixture(scope="module")
def golden():
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


def test_oracle_reproduces_the_golden_vectors(oracle, golden):
    now = make_golden.compute(oracle, golden)
    assert sorted(now) == sorted(golden)
    for k, v in golden.items():
        if v.dtype.names:
            for f in v.dtype.names:
                np.testing.assert_array_equal(now[k][f], v[f], err_msg=f"{k}.{f}")
        else:
            np.testing.assert_array_equal(now[k], v, err_msg=k)


@pytest.mark.gpu
def test_gpu_matches_the_golden_vectors(gpu, oracle, golden):
    """Same bars as the live GPU-vs-oracle parity tests: closest hits agree on ids (or tie
    within 1e-6 relative distance) and on t within 1e-5; BSDF values within 1e-5 / 1e-6;
    display-film weights exact and colours equal at 99% of pixels; tree hashes exact.

    The scenes are generated by numpy, whose transcendental functions may round
    differently on another CPU; when this host's oracle does not reproduce the file,
    the scenes differ and the comparison is skipped (the live parity tests still run)."""
    ref = make_golden.compute(oracle, golden)
    if any(not np.array_equal(ref[k], golden[k]) for k in golden):
        pytest.skip("the scene generators round differently on this host")
    now = make_golden.compute(gpu, golden)
    for name in ("cornell_hits", "disp_hits"):
        hg, ho = now[name], golden[name]
        assert ((hg["prim"] >= 0) == (ho["prim"] >= 0)).all(), name
        both = (hg["prim"] >= 0) & (ho["prim"] >= 0)
        same = (hg["prim"] == ho["prim"]) & (hg["component"] == ho["component"])
        tie = np.abs(hg["t"] - ho["t"]) <= 1e-6 * np.abs(ho["t"])
        assert (both & ~same & ~tie).sum() == 0, name
        np.testing.assert_allclose(hg["t"][both & same], ho["t"][both & same], rtol=1e-5, err_msg=name)
    for k in golden:
        if k.startswith(("bsdf_f_", "bsdf_pdf_")):
            np.testing.assert_allclose(now[k], golden[k], rtol=1e-5, atol=1e-6, err_msg=k)
    np.testing.assert_array_equal(now["display_weight"], golden["display_weight"])
    assert (now["display_accum"] == golden["display_accum"]).all(axis=-1).mean() > 0.99
    np.testing.assert_array_equal(now["tree_hash"], golden["tree_hash"])
