"""netchem on the GPU: node centres of mass computed by the device kernel
from raw DCD frames, against the oracle's restatement of
netchem/src/network.cpp (bit-exact), the reference's stride expectations,
and the device-resident coordinates feeding the KSG entry points."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _files(tmp_path, n_res=40, n_frames=23, seed=11, **kw):
    from netsci_gb300 import synthetic
    dcd, pdb, _ = synthetic.protein_files(tmp_path, n_res, n_frames, seed=seed, **kw)
    return dcd, pdb


@pytest.mark.parametrize("kw", [dict(), dict(big_endian=True), dict(marker_bytes=8),
                                dict(charmm=False), dict(four_dims=True, unit_cell=False)])
def test_node_coordinates_match_oracle(oracle_mod, tmp_path, kw):
    from netsci_gb300 import netchem
    dcd, pdb = _files(tmp_path, **kw)
    net = netchem.Network()
    net.init(dcd, pdb, 0, 22, 1)
    X, nodes = oracle_mod.node_coordinates(dcd, pdb, 0, 22, 1)
    assert net.numNodes() == len(nodes) == 40 and net.numFrames() == 23
    got = net.nodeCoordinates().toNumpy2D()
    assert got.shape == X.shape and np.array_equal(got, X)
    for n, (tag, members, tm) in zip(net.nodes(), nodes):
        assert n.tag() == tag and n.numAtoms() == len(members) and n.totalMass() == tm
        assert [a.index() for a in n.atoms()] == members
        assert n.hash() == 0
    assert net.nodeFromAtomIndex(nodes[3][1][0]).index() == 3


@pytest.mark.parametrize("first,last,stride", [(0, 22, 2), (0, 22, 3), (5, 17, 4), (3, -1, 1),
                                               (22, 22, 1)])
def test_frame_selection(oracle_mod, tmp_path, first, last, stride):
    from netsci_gb300 import netchem
    dcd, pdb = _files(tmp_path)
    net = netchem.Network()
    net.init(dcd, pdb, first, last, stride)
    X, _ = oracle_mod.node_coordinates(dcd, pdb, first, last, stride)
    assert np.array_equal(net.nodeCoordinates().toNumpy2D(), X)


def test_stride_coordinate_equality(tmp_path):
    """The reference's stride tests (tests/netchem/python/test_Network.py):
    stride-s frame j equals stride-1 frame s*j, per plane."""
    from netsci_gb300 import netchem
    dcd, pdb = _files(tmp_path, n_frames=10)
    full = netchem.Network()
    full.init(dcd, pdb, 0, 9)
    X1 = full.nodeCoordinates().toNumpy2D()
    for s in (1, 2, 3):
        net = netchem.Network()
        net.init(dcd, pdb, 0, 9, s)
        m = net.numFrames()
        assert m == len(range(0, 10, s))
        Xs = net.nodeCoordinates().toNumpy2D()
        for c in range(3):
            assert np.array_equal(Xs[:, c * m:(c + 1) * m], X1[:, c * 10:(c + 1) * 10][:, ::s])


def test_many_frames_batches(oracle_mod, tmp_path):
    """Enough frames for several staging batches (frames > 64 MB / frame size)."""
    from netsci_gb300 import netchem, synthetic
    dcd, pdb, _ = synthetic.protein_files(tmp_path, 600, 1600, seed=2)
    net = netchem.Network()
    net.init(dcd, pdb, 0, -1, 1)
    X, _ = oracle_mod.node_coordinates(dcd, pdb, 0, -1, 1)
    assert np.array_equal(net.nodeCoordinates().toNumpy2D(), X)


def test_device_coordinates_feed_ksg(tmp_path):
    """GC from the device-resident coordinates equals GC through the host
    CuArray API on the same network."""
    import netcalc
    import cuarray
    from netsci_gb300 import device, netchem, synthetic
    dcd, pdb = _files(tmp_path, n_res=12, n_frames=300)
    net = netchem.Network()
    net.init(dcd, pdb, 0, -1)
    Xd, m = net.deviceCoordinates()
    assert Xd.shape[0] == 12 and Xd.shape[1] == 3 and Xd.shape[2] % 64 == 0 and m == 300
    assert torch.isinf(Xd[:, :, m:]).all()
    ab = synthetic.all_pairs(12)
    pairs = device.make_pairs(Xd, m, ab)
    mi = torch.empty(len(pairs), device="cuda")
    device.ksg_pairs(pairs, 6, 3, mi=mi)
    R = cuarray.FloatCuArray()
    AB = cuarray.IntCuArray()
    AB.fromNumpy2D(ab.astype(np.int32))
    I = cuarray.FloatCuArray()
    netcalc.mutualInformation(net.nodeCoordinates(), I, AB, 6, m, 2, 3, netcalc.GPU_PLATFORM)
    assert np.array_equal(mi.cpu().numpy(), I.toNumpy1D())


def test_init_errors(tmp_path):
    from netsci_gb300 import NsgError, netchem, synthetic
    dcd, pdb = _files(tmp_path)
    net = netchem.Network()
    with pytest.raises(NsgError) as e:
        net.init(dcd, pdb, 0, 23, 1)           # past the last frame
    assert e.value.status == 1
    (tmp_path / "b").mkdir()
    other, _, _ = synthetic.protein_files(tmp_path / "b", 7, 3, seed=1)
    with pytest.raises(NsgError) as e:
        net.init(other, pdb, 0, 2, 1)          # atom counts differ
    assert e.value.status == 1
    net.init(dcd, pdb, 0, 4, 1)               # still usable afterwards
    assert net.numFrames() == 5
