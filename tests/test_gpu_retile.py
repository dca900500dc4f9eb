"""Device-side retile of spin-orbital tile blocks (ccsdt_upload_begin / blocks / end): blocks laid
out as ExaChem's Tensor::get returns them (row-major in the tensor's index order, the index maps
of the C++ adapter's gather) must give the same inputs - and so bit-identical energies - as
ccsdt_upload of the spatial arrays."""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OCC, VIR = [4, 5], [16, 16, 18]


def _offsets(ext):
    return np.concatenate([[0], np.cumsum(ext)[:-1]]).astype(int)


def _blocks(d, kind):
    """(tiles, offsets, data) of every block of one tensor, in the block layouts of ccsdt.h."""
    oo, vo = _offsets(OCC), _offsets(VIR)
    O = lambda t: slice(oo[t], oo[t] + OCC[t])
    V = lambda t: slice(vo[t], vo[t] + VIR[t])
    no, nv = len(OCC), len(VIR)
    tiles, parts = [], []
    if kind == "t2":      # (A, B, I, J): [a][b][i][j] <- t2[i][j][a][b]
        for A, B, I, J in itertools.product(range(nv), range(nv), range(no), range(no)):
            tiles.append((A, B, I, J)); parts.append(d["t2"][O(I), O(J), V(A), V(B)].transpose(2, 3, 0, 1))
    elif kind == "oovv":  # (I, J, A, B): [i][j][a][b]
        for I, J, A, B in itertools.product(range(no), range(no), range(nv), range(nv)):
            tiles.append((I, J, A, B)); parts.append(d["oovv"][O(I), O(J), V(A), V(B)])
    elif kind == "ooov":  # (I, K, J, A): [i][k][j][a] <- ooov[i][j][k][a]
        for I, K, J, A in itertools.product(range(no), range(no), range(no), range(nv)):
            tiles.append((I, K, J, A)); parts.append(d["ooov"][O(I), O(J), O(K), V(A)].transpose(0, 2, 1, 3))
    else:                 # (I, B, A, C): [i][b][a][c] <- ovvv[i][a][b][c]
        for I, B, A, C in itertools.product(range(no), range(nv), range(nv), range(nv)):
            tiles.append((I, B, A, C)); parts.append(d["ovvv"][O(I), V(A), V(B), V(C)].transpose(0, 2, 1, 3))
    flat = [np.ascontiguousarray(p).ravel() for p in parts]
    offs = np.concatenate([[0], np.cumsum([f.size for f in flat])[:-1]])
    return np.array(tiles), offs, np.concatenate(flat)


def test_retiled_blocks_equal_spatial_upload(built):
    import torch
    from exachem_gb300.ccsd_t import FusedTriples
    from exachem_gb300.generator import generate
    o, v = sum(OCC), sum(VIR)
    d = generate(o, v, 61)
    ref = FusedTriples(o, v, OCC, VIR)
    ref.upload_dict(d)
    r64, r3 = ref.energy("fp64"), ref.energy("ozaki", slices=3)
    ft = FusedTriples(o, v, OCC, VIR)
    ft.upload_begin(d["eps_occ"], d["eps_vir"], d["t1"])
    for kind in ("t2", "oovv", "ooov", "ovvv"):
        tiles, offs, data = _blocks(d, kind)
        half = len(tiles) // 2          # several calls per tensor; the second from device memory
        ft.upload_blocks(kind, tiles[:half], offs[:half], data)
        rest = torch.from_numpy(data[offs[half]:]).cuda()
        ft.upload_blocks(kind, tiles[half:], offs[half:] - offs[half], rest)
    ft.upload_end()
    g64, g3 = ft.energy("fp64"), ft.energy("ozaki", slices=3)
    assert g64["e_paren_T"] == r64["e_paren_T"] and g64["e_bracket_T"] == r64["e_bracket_T"]
    assert g3["e_paren_T"] == r3["e_paren_T"]


def test_retile_rejects_bad_blocks(built):
    from exachem_gb300.ccsd_t import CCSDTError, FusedTriples
    from exachem_gb300.generator import generate
    o, v = sum(OCC), sum(VIR)
    d = generate(o, v, 62)
    ft = FusedTriples(o, v, OCC, VIR)
    with pytest.raises(CCSDTError):      # blocks before ccsdt_upload_begin
        ft.upload_blocks("oovv", [(0, 0, 0, 0)], [0], np.zeros(OCC[0] ** 2 * VIR[0] ** 2))
    ft.upload_begin(d["eps_occ"], d["eps_vir"], d["t1"])
    with pytest.raises(CCSDTError):      # virtual tile index outside the layout
        ft.upload_blocks("oovv", [(0, 0, 0, 3)], [0], np.zeros(10 ** 5))
    with pytest.raises(CCSDTError):      # block past the end of the data
        ft.upload_blocks("oovv", [(0, 0, 0, 0)], [5], np.zeros(OCC[0] ** 2 * VIR[0] ** 2))
    with pytest.raises(CCSDTError):      # energy before ccsdt_upload_end
        ft.energy("fp64")
