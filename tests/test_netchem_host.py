"""netchem host side: the DCD reader, PDB parsing and the oracle's
restatement, pinned against the reference's own DCD plugin and Atom class
(compiled into oracle/_ref when the reference sources are present) on the
reference's test and tutorial trajectories and on synthetic files in every
DCD variant (byte order, record-marker width, CHARMM / X-PLOR, unit cell,
fourth dimension)."""
import os
from pathlib import Path

import numpy as np
import pytest

REF = Path(os.environ.get("NETSCI_REF", str(Path(__file__).resolve().parent.parent / "baseline" / "_ref" / "netsci")))
REF_FILES = [
    (REF / "tests/netchem/cpp/data/test.dcd", REF / "tests/netchem/cpp/data/test.pdb"),
    (REF / "tutorial/protG_short.dcd", REF / "tutorial/protG_short.pdb"),
]

VARIANTS = [
    dict(),
    dict(big_endian=True),
    dict(unit_cell=False),
    dict(charmm=False),
    dict(four_dims=True),
    dict(marker_bytes=8),
    dict(marker_bytes=8, big_endian=True),
]


def _ref_or_skip(oracle_mod):
    if oracle_mod.ref_netchem() is None or not REF_FILES[0][0].exists():
        pytest.skip("reference netchem sources not available")


@pytest.mark.parametrize("pair", REF_FILES, ids=["test", "protG_short"])
def test_oracle_dcd_reader_matches_reference_plugin(oracle_mod, pair):
    _ref_or_skip(oracle_mod)
    ref = oracle_mod.ref_dcd_frames(pair[0])
    _, mine = oracle_mod.dcd_read(pair[0])
    assert mine.shape == ref.shape and np.array_equal(mine, ref)


@pytest.mark.parametrize("kw", [v for v in VARIANTS if v.get("marker_bytes", 4) == 4
                                and not (v.get("big_endian") and v.get("four_dims"))])
def test_oracle_dcd_reader_matches_plugin_on_variants(oracle_mod, tmp_path, kw):
    _ref_or_skip(oracle_mod)
    from netsci_gb300 import synthetic
    dcd, _, frames = synthetic.protein_files(tmp_path, 12, 5, seed=3, **kw)
    assert np.array_equal(oracle_mod.ref_dcd_frames(dcd), frames)
    assert np.array_equal(oracle_mod.dcd_read(dcd)[1], frames)


@pytest.mark.parametrize("kw", VARIANTS)
def test_library_dcd_reader_matches_oracle(oracle_mod, tmp_path, kw):
    from netsci_gb300 import netchem, synthetic
    dcd, _, frames = synthetic.protein_files(tmp_path, 15, 9, seed=5, **kw)
    assert netchem.dcd_info(dcd) == (frames.shape[2], 9)
    assert np.array_equal(netchem.dcd_read(dcd), frames)
    assert np.array_equal(netchem.dcd_read(dcd, 1, 3, 3), frames[1:8:3])


@pytest.mark.parametrize("pair", REF_FILES, ids=["test", "protG_short"])
def test_library_dcd_reader_on_reference_files(oracle_mod, pair):
    _ref_or_skip(oracle_mod)
    from netsci_gb300 import netchem
    assert np.array_equal(netchem.dcd_read(pair[0]), oracle_mod.ref_dcd_frames(pair[0]))


def _pdb_paths(tmp_path):
    from netsci_gb300 import synthetic
    _, pdb, _ = synthetic.protein_files(tmp_path, 30, 2, seed=9)
    return [p for _, p in REF_FILES] + [Path(pdb)]


def test_pdb_parsing_matches_reference_atom(oracle_mod, tmp_path):
    _ref_or_skip(oracle_mod)
    from netsci_gb300 import netchem
    for pdb in _pdb_paths(tmp_path):
        mass, resid, h, tags, els, names = oracle_mod.ref_pdb_atoms(pdb)
        mine = oracle_mod.pdb_atoms(pdb)
        assert len(mine) == len(mass)
        assert np.array_equal(np.array([a["mass"] for a in mine], np.float32), mass)
        assert [a["residueId"] for a in mine] == resid.tolist()
        assert [a["hash"] for a in mine] == h.tolist()
        assert [a["tag"] for a in mine] == tags
        assert [a["element"] for a in mine] == els
        assert [a["name"] for a in mine] == names
        net = netchem.Network()
        net.parsePdb(pdb)
        lib_atoms = list(net.atoms())
        assert len(lib_atoms) == len(mass)
        assert np.array_equal(np.array([a.mass() for a in lib_atoms], np.float32), mass)
        assert [a.hash() for a in lib_atoms] == h.tolist()
        assert [a.tag() for a in lib_atoms] == tags
        assert [a.element() for a in lib_atoms] == els


def test_weight_table_matches_reference(oracle_mod, tmp_path):
    """Every element of the reference's table (and one it lacks) through the
    reference's Atom, the oracle and the library."""
    _ref_or_skip(oracle_mod)
    import re
    from netsci_gb300 import netchem, synthetic
    text = (REF / "netchem/include/chemical_properties.h").read_text()
    table = dict(re.findall(r'\{"([A-Za-z]+)",\s*([0-9.]+)\}', text))
    assert len(table) == len(oracle_mod._ATOMIC_WEIGHTS_G)
    for el, v in table.items():
        assert float(v) == oracle_mod.atomic_weight_kg(el), el
    els = list(table) + ["V"]
    atoms = [dict(name="X", resname="UNK", chain="A", resid=i + 1, x=0.0, y=0.0, z=0.0,
                  occupancy=1.0, segment="S", element=e.upper()) for i, e in enumerate(els)]
    pdb = tmp_path / "elements.pdb"
    synthetic.write_pdb(pdb, atoms)
    ref_mass = oracle_mod.ref_pdb_atoms(pdb)[0]
    net = netchem.Network()
    net.parsePdb(pdb)
    lib_mass = np.array([a.mass() for a in net.atoms()], np.float32)
    ora_mass = np.array([a["mass"] for a in oracle_mod.pdb_atoms(pdb)], np.float32)
    assert np.array_equal(lib_mass, ref_mass) and np.array_equal(ora_mass, ref_mass)
    assert lib_mass[-1] == 0.0   # vanadium is not in the table


def test_oracle_node_coordinates_reference_counts(oracle_mod):
    """The reference's own expectations for its test trajectory
    (tests/netchem/cpp/NetworkStride{1,2,3}_test.cpp): 290 nodes; 10, 5 and 4
    frames for strides 1, 2, 3 over frames 0..9; stride s frame j equals
    stride 1 frame s*j (tests/netchem/python/test_Network.py)."""
    _ref_or_skip(oracle_mod)
    dcd, pdb = REF_FILES[0]
    X1, nodes = oracle_mod.node_coordinates(dcd, pdb, 0, 9, 1)
    assert len(nodes) == 290 and X1.shape == (290, 30)
    for s, m in ((2, 5), (3, 4)):
        Xs, _ = oracle_mod.node_coordinates(dcd, pdb, 0, 9, s)
        assert Xs.shape == (290, 3 * m)
        for c in range(3):
            assert np.array_equal(Xs[:, c * m:(c + 1) * m], X1[:, c * 10:(c + 1) * 10][:, ::s])


def test_pdb_errors():
    from netsci_gb300 import NsgError, netchem
    net = netchem.Network()
    with pytest.raises(NsgError) as e:
        net.parsePdb("/nonexistent/file.pdb")
    assert e.value.status == 6
    with pytest.raises(NsgError) as e:
        netchem.dcd_info("/nonexistent/file.dcd")
    assert e.value.status == 6
