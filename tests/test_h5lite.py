"""HDF5-subset reader/writer: the reference's own example config and a round trip."""
import os

import numpy as np

from conftest import GOLDEN


def test_reads_reference_config(built):
    from h5lite import H5File
    f = H5File(os.path.join(GOLDEN, "chig.up"))
    assert f.read("/input/pos").shape == (30, 3, 1)
    assert [s.decode() for s in f.read("/input/sequence")][:3] == ["GLY", "TYR", "ASP"]
    # chunked + shuffle + deflate + fletcher32 dataset
    eq = f.read("/input/potential/Spring_bond/equil_dist")
    assert np.allclose(eq[:3], [1.453, 1.526, 1.3])
    names = f.list("/input/potential")
    assert "rotamer" in names and "affine_alignment" in names
    args = f.attr("/input/potential/rotamer", "arguments")
    assert [a.decode() for a in args][0] == "placement_fixed_point_vector_only"
    assert f.read("/input/potential/rotamer/pair_interaction/interaction_param").shape == (20, 20, 54)
    assert abs(float(f.attr("/input/potential/rotamer", "damping")) - 0.4) < 1e-12


def test_writer_round_trip(built, tmp_path):
    from h5lite import H5File, H5Writer
    w = H5Writer()
    a = np.arange(24, dtype=np.float64).reshape(2, 3, 4)
    w.dataset("/g/sub/a", a)
    w.dataset("/g/i", np.array([1, -2, 3], np.int32))
    w.dataset("/g/s", np.array([b"pos", b"affine"]))
    w.set_attr("/g", "scalar", 7)
    w.set_attr("/g", "names", np.array([b"x", b"yy"]))
    w.set_attr("/g/sub/a", "f", 0.25)
    for k in range(40):  # many links in one group
        w.dataset("/many/n%02d" % k, np.array([k]))
    p = str(tmp_path / "t.h5")
    w.save(p)
    f = H5File(p)
    assert np.array_equal(f.read("/g/sub/a"), a)
    assert np.array_equal(f.read("/g/i"), [1, -2, 3])
    assert [x.decode() for x in f.read("/g/s")] == ["pos", "affine"]
    assert int(f.attr("/g", "scalar")) == 7
    assert [x.decode() for x in f.attr("/g", "names")] == ["x", "yy"]
    assert float(f.attr("/g/sub/a", "f")) == 0.25
    assert f.list("/many") == ["n%02d" % k for k in range(40)]
    assert int(f.read("/many/n37")[0]) == 37


def test_missing_and_corrupt(built, tmp_path):
    import pytest
    from h5lite import H5File
    with pytest.raises(IOError):
        H5File(str(tmp_path / "nope.h5"))
    bad = tmp_path / "bad.h5"
    bad.write_bytes(b"not an hdf5 file at all" * 10)
    with pytest.raises(IOError):
        H5File(str(bad))
    # truncated copy of a real file: reading objects must fail cleanly
    data = open(os.path.join(GOLDEN, "chig.up"), "rb").read()
    tr = tmp_path / "trunc.up"
    tr.write_bytes(data[:4096])
    try:
        f = H5File(str(tr))
    except IOError:
        return
    with pytest.raises(KeyError):
        f.read("/input/potential/rotamer/pair_interaction/interaction_param")
