"""Readers of distance tables, NEXUS location annotations and BEAST logs
(massivemds_gb300/formats.py), on small files written here, plus the H3N2
fixture of the reference when it is present."""
import numpy as np
import pytest

from massivemds_gb300 import formats
from tests import kat


def test_distance_table_with_missing_cells(tmp_path):
    p = tmp_path / "d.txt"
    p.write_text("\ta\tb\tc\n" "a\t0\t1.5\tNA\n" "c\t\t2\t0\n" "b\t1.5\t0\t2\t\n")
    names, d = formats.read_distance_table(str(p))
    assert names == ["a", "b", "c"]
    assert d[0, 1] == 1.5 and np.isnan(d[0, 2]) and np.isnan(d[2, 0])
    assert d[1, 2] == 2.0 and d[2, 1] == 2.0 and d[1, 1] == 0.0


def test_nexus_locations_and_log(tmp_path):
    t = tmp_path / "x.trees"
    t.write_text("#NEXUS\nBegin trees;\n\tTranslate\n\t\t1 alpha,\n\t\t2 'beta',\n\t\t3 gamma\n\t\t;\n"
                 "tree STATE_0 = ((1[&rate=1,loc={0.5,-1.0,2}]:1,2[&loc={1.5,2.5,3}]:1):1,3[&loc={0,0,1e-3}]:2);\n"
                 "tree STATE_10 = ((1[&loc={9,8,7}]:1,2[&loc={6,5,4}]:1):1,3[&loc={3,2,1}]:2);\nEnd;\n")
    st, locs = formats.read_nexus_locations(str(t), state=0)
    assert st == 0 and np.allclose(locs["alpha"], [0.5, -1.0, 2]) and np.allclose(locs["gamma"], [0, 0, 1e-3])
    st, locs = formats.read_nexus_locations(str(t))
    assert st == 10 and np.allclose(locs["beta"], [6, 5, 4])
    x = formats.locations_in_order(["gamma", "alpha"], locs)
    assert x.shape == (2, 3) and np.allclose(x[0], [3, 2, 1])
    with pytest.raises(KeyError):
        formats.locations_in_order(["delta"], locs)
    lg = tmp_path / "x.log"
    lg.write_text("# comment\nstate\tprec\tlik\n0\t1.5\t-10.0\n10\t2.5\t-9.5\n")
    assert formats.read_beast_log(str(lg), ["prec", "lik"], 10) == {"prec": 2.5, "lik": -9.5}


@pytest.mark.skipif(not kat.available(), reason="reference fixtures not present")
def test_h3n2_fixture_reads():
    delta, x, tau, logged = kat.load_state()
    assert delta.shape == (372, 372) and x.shape == (372, 2)
    assert np.allclose(delta, delta.T) and np.all(np.diag(delta) == 0) and not np.isnan(delta).any()
    assert tau > 0 and logged < 0
