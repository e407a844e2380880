"""Drop-in parameter-file reader and array normalisation against the
reference's outputs (tests/golden/support.npz, made by running the
reference's Support.ReadParameters / NormalizeArray on these lines)."""

import numpy as np
import pytest

from conftest import golden


def test_read_parameters_types_every_line_as_the_reference(tmp_path):
    from opensss_gb300.Support import ReadParameters

    g = golden("support")
    path = tmp_path / "params.txt"
    path.write_text("\n".join(str(x) for x in g["lines"]) + "\n")
    assert repr(ReadParameters(str(path))) == str(g["params_repr"])


def test_read_parameters_rejects_what_the_reference_rejects(tmp_path):
    from opensss_gb300.Support import ReadParameters

    g = golden("support")
    path = tmp_path / "params.txt"
    for line, err in zip(g["bad_lines"], g["bad_errors"]):
        path.write_text(str(line) + "\n")
        with pytest.raises({"ValueError": ValueError, "IndexError": IndexError}[str(err)]):
            ReadParameters(str(path))


@pytest.mark.parametrize("i", range(4))
def test_normalize_array_matches_reference(i):
    from opensss_gb300.Support import NormalizeArray

    g = golden("support")
    lo, hi = (float(v) for v in g[f"normalize{i}_range"])  # ints in the reference call; the same values
    got = NormalizeArray(g[f"normalize{i}_in"], lo, hi)
    ref = g[f"normalize{i}"]
    assert got.dtype == ref.dtype and np.array_equal(got, ref)
