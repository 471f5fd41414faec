"""The comparison helpers the parity tests rely on: a NaN or infinite field
component must never pass by comparisons that are false for NaN."""
import warnings

import numpy as np

from helpers import field_close, max_rel_err


def test_non_finite_components_must_match_position_by_position():
    ref = np.array([[complex(np.inf, np.nan), 1 + 1j, 0j], [1 + 0j, 2 + 0j, 3 + 0j]])
    with warnings.catch_warnings():
        warnings.simplefilter("error", RuntimeWarning)
        assert field_close(ref.copy(), ref) == []
        assert max_rel_err(ref, ref) == 0.0
        finite = ref.copy()
        finite[0, 0] = 1 + 0j
        assert [b[4] for b in field_close(finite, ref)] == ["non-finite"]
        assert [b[4] for b in field_close(ref, finite)] == ["non-finite"]
        swapped = ref.copy()
        swapped[0, 0] = complex(-np.inf, np.nan)
        assert [b[4] for b in field_close(swapped, ref)] == ["non-finite"]
        nan_both = ref.copy()
        nan_both[0, 0] = complex(np.nan, np.nan)
        assert field_close(nan_both, ref)


def test_finite_tolerance():
    ref = np.array([[1 + 0j, 1j, 0j]])
    assert field_close(ref * (1 + 5e-5), ref) == []
    assert field_close(ref * (1 + 2e-4), ref)
    assert field_close(ref * np.exp(2e-3j), ref)
