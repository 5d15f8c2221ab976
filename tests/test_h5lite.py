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


def _walk(f, path="/"):
    out = []
    for k in f.list(path):
        q = path.rstrip("/") + "/" + k
        out.append(q)
        if f.kind(q) == 1:
            out += _walk(f, q)
    return out


def test_cpp_writer_copies_reference_config_exactly(built, tmp_path):
    """The C++ writer the upside driver logs with rewrites the reference's own
    PyTables-written config: every dataset and attribute byte for byte
    (datasets come back contiguous and uncompressed), PyTables' empty TITLE
    attributes (null dataspaces) included, and skipped paths left out."""
    import h5lite
    from h5lite import H5File
    src = os.path.join(GOLDEN, "chig.up")
    dst = str(tmp_path / "copy.up")
    h5lite.copy_file(src, dst, ["/input/potential/rama_map_pot"])
    a, b = H5File(src), H5File(dst)
    pa, pb = _walk(a), _walk(b)
    assert set(pa) - set(pb) == {"/input/potential/rama_map_pot"} | {
        p for p in pa if p.startswith("/input/potential/rama_map_pot/")}
    assert set(pb) <= set(pa)
    n = 0
    for q in pb + ["/"]:
        if q != "/" and a.kind(q) == 0:
            x, y = a.read(q), b.read(q)
            assert x.dtype == y.dtype and x.shape == y.shape and x.tobytes() == y.tobytes(), q
            n += 1
        ax, bx = a.attrs(q), b.attrs(q)
        assert set(ax) == set(bx), q
        for k in ax:
            if ax[k] is None:
                assert bx[k] is None, (q, k)
            else:
                assert np.asarray(ax[k]).tobytes() == np.asarray(bx[k]).tobytes(), (q, k)
    assert n > 100
    # and a file the Python writer made, scalars and strings included
    w = h5lite.H5Writer()
    w.dataset("/s/f", np.float32(2.5))
    w.dataset("/s/u", np.arange(5, dtype=np.uint16))
    w.dataset("/s/names", np.array([b"ab", b"cde"]))
    w.set_attr("/s", "k", np.array([1, 2, 3], np.int64))
    p1, p2 = str(tmp_path / "p1.h5"), str(tmp_path / "p2.h5")
    w.save(p1)
    h5lite.copy_file(p1, p2)
    c = H5File(p2)
    assert float(c.read("/s/f")) == 2.5 and c.read("/s/f").shape == ()
    assert c.read("/s/u").dtype == np.uint16 and list(c.read("/s/u")) == [0, 1, 2, 3, 4]
    assert [x.decode() for x in c.read("/s/names")] == ["ab", "cde"]
    assert list(c.attr("/s", "k")) == [1, 2, 3]
