"""Host-side parts of the restart / time-history surface (no GPU needed)."""
import pytest

import immerseflow_gb300 as ifx
from immerseflow_gb300 import _capi as capi


def test_probe_file_grammar(tmp_path):
    """probe_init (test/UTIL_PRE_SIM.f90:172-202): count, a skipped line, "x y" per probe."""
    f = tmp_path / "probe.dat"
    f.write_text("3\nx  y\n1.5 2.0\n  -0.25   7\n3.0,4.5\n")
    xy = ifx.probes_read(str(f))
    assert xy.tolist() == [[1.5, 2.0], [-0.25, 7.0], [3.0, 4.5]]
    f.write_text("0\n\n")
    assert ifx.probes_read(str(f)).shape == (0, 2)


@pytest.mark.parametrize("text", ["two\n\n1 2\n", "2\nskip\n1 2\n", "1\nskip\n1\n"])
def test_probe_file_errors(tmp_path, text):
    f = tmp_path / "probe.dat"
    f.write_text(text)
    with pytest.raises(ifx.IFXError) as e:
        ifx.probes_read(str(f))
    assert e.value.status == capi.IFX_ERR_PARSE


def test_probe_file_missing(tmp_path):
    with pytest.raises(ifx.IFXError) as e:
        ifx.probes_read(str(tmp_path / "none.dat"))
    assert e.value.status == capi.IFX_ERR_IO
