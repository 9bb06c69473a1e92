"""Binary force-constant (full-Hamiltonian) phonon path over the C ABI.

The reference's ``qe_fc = 0`` branch reads a binary force-constant matrix of
the whole sandwich (negf/fc.f90:11-44), builds reduced index tables once
(gen_fc_to_dyn_idx, negf/dyn.f90:988-1093, flattened as
negf/phinfortran.f90:655-683), partitions the device part of the dense D(q)
into layers (blockwise_setup, negf/device.f90:11-249) and then, per
transverse k, builds the dense D(q) (gen_dyn, negf/dyn.f90:39-150) and runs
surface_green (negf/surface.f90:118-342) and G_block (negf/device.f90:289-560)
on slices of it (negf/phinfortran.f90:929-960).

Here the set-up (tables, partition) runs once on the host, and per call the
dense D(q) of every k is built on the GPU (``pf_gen_dyn_dev``), sliced into
the block set of the tdb transport entries on the GPU
(``pf_dense_to_tdb_dev``), and solved by the same transport engine as the
tdb path: surface_green/G_block compute the same lead decimations, device
sweep and Caroli trace as surface_green_tdb/get_G_full_tdb on those slices
(same device factor 10, same wrapper conversions, negf/device.f90:280-285).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi
from .transport import BLOCK_NAMES

TOL = 1.0e-7   # blockwise_setup's sparsity threshold (negf/device.f90:43-131)


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def central_start(n_uc, nx, ny, nz):
    """0-based first fc column atom of the central supercell cell."""
    return n_uc * (nx * (2 * ny + 1) * (2 * nz + 1) + ny * (2 * nz + 1) + nz)


def row_atoms(natoms, nbx, nby, n_uc, nz):
    """fc row atom of every structure atom (negf/dyn.f90:95-103)."""
    per = n_uc // nz
    a = np.arange(natoms)
    iz = a // (nby * nbx * per)
    rem = a - iz * nby * nbx * per
    rem = rem - (rem // (nbx * per)) * nbx * per
    return (iz * per + rem % per).astype(np.int32)


@dataclass
class FcTables:
    """Reduced index tables: entries of every atom pair in (a, b) row-major
    order (num[a, b] each), 0-based fc column atom and bond vector."""
    num: np.ndarray   # (natoms, natoms) int
    idx: np.ndarray   # (nent,) int, 0-based
    dr: np.ndarray    # (nent, 3) Angstrom

    def pairs(self):
        """(pair_a, pair_b, pair_off) of the atom pairs with entries."""
        a, b = np.nonzero(self.num)
        cnt = self.num[a, b]
        off = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int32)
        return a.astype(np.int32), b.astype(np.int32), off


def fc_tables(pos_sc, pos, cell, nbx, nby, n_uc, nz, nfc, r_cutoff, lead=False):
    """Index tables of gen_fc_to_dyn_idx (lead=False, negf/dyn.f90:988-1093)
    or gen_lead_fc_to_dyn_idx (lead=True, :1095-1216; returns the in-layer and
    the coupling tables).  For every atom pair and each of the 27 structure
    images (dx, dy, dz) inside r_cutoff, the fc supercell atoms sitting at the
    same bond vector (within 1e-3) are the entries, in ascending fc order."""
    from scipy.spatial import cKDTree
    nx, ny, nzf = nfc
    pos_sc = np.asarray(pos_sc, dtype=np.float64)[:, :3]
    pos = np.asarray(pos, dtype=np.float64)[:, :3]
    cell = np.asarray(cell, dtype=np.float64)
    natoms = pos.shape[0]
    i0 = central_start(n_uc, nx, ny, nzf)
    ncell = (2 * nx + 1) * (2 * ny + 1) * (2 * nzf + 1)
    cell_of = np.arange(pos_sc.shape[0]) // n_uc
    kk_of = cell_of % (2 * nzf + 1)
    if lead:
        groups = [np.nonzero(kk_of == nzf)[0], np.nonzero(kk_of == 2 * nzf)[0]]
        fc_row = np.arange(natoms) % n_uc          # negf/dyn.f90:1177-1181
    else:
        groups = [np.arange(ncell * n_uc)]
        fc_row = row_atoms(natoms, nbx, nby, n_uc, nz)
    trees = [cKDTree(pos_sc[g]) for g in groups]
    shifts = np.array([[dx, dy, dz] for dx in (-1, 0, 1) for dy in (-1, 0, 1) for dz in (-1, 0, 1)],
                      dtype=np.float64) @ cell
    out = []
    for g, tree in zip(groups, trees):
        num = np.zeros((natoms, natoms), dtype=np.int64)
        ent = {}
        for a in range(natoms):
            i = i0 + fc_row[a]
            dr = pos[None, :, :] + shifts[:, None, :] - pos[a][None, None, :]      # (27, natoms, 3)
            ok = np.sqrt(np.einsum("sbc,sbc->sb", dr, dr)) < r_cutoff
            for s, b in zip(*np.nonzero(ok)):
                hits = tree.query_ball_point(pos_sc[i] + dr[s, b], 1.0e-3)
                if not hits:
                    continue
                # the reference's test is |pos_sc[idx] - pos_sc[i] - dr| < 1e-3
                cand = np.sort(g[np.asarray(hits)])
                d = pos_sc[cand] - pos_sc[i] - dr[s, b]
                cand = cand[np.sqrt(np.einsum("ij,ij->i", d, d)) < 1.0e-3]
                ent.setdefault((a, b), []).extend((int(c), dr[s, b]) for c in cand)
                num[a, b] += cand.size
        keys = sorted(ent)
        idx = np.array([c for k in keys for c, _ in ent[k]], dtype=np.int64)
        drs = np.array([d for k in keys for _, d in ent[k]], dtype=np.float64).reshape(-1, 3)
        out.append(FcTables(num, idx, drs))
    return out if lead else out[0]


def blockwise_setup(H, nl, nr, n_buffer_l, n_buffer_r):
    """Layer sizes of the device part of a dense matrix by the partition rule
    of negf/device.f90:11-249: the first layer reaches the last column the
    left lead cell couples to; each further layer is as short as the
    sparsity allows (its couplings beyond the next layer vanish below 1e-7);
    the remainder forms the last layer, merged into the previous ones while
    it is shorter than the right lead cell's reach."""
    A = np.abs(np.asarray(H)) > TOL
    norb = A.shape[0]
    nd = norb - n_buffer_l - n_buffer_r - 2 * nl - 2 * nr
    if nd < 2:
        raise ValueError("blockwise_setup: device part too small")
    d0 = n_buffer_l + 2 * nl
    # reach of the left cell into the device: last nonzero column (1-based) of
    # each row, counting only rows whose last nonzero is before column nd
    VLD = A[n_buffer_l + nl:n_buffer_l + 2 * nl, d0:d0 + nd]
    maxij1 = 0
    for row in VLD:
        nz = np.nonzero(row)[0]
        if nz.size and nz[-1] + 1 <= nd - 1:
            maxij1 = max(maxij1, int(nz[-1]) + 1)
    VRD = A[norb - n_buffer_r - 2 * nr:norb - n_buffer_r - nr, norb - n_buffer_r - 2 * nr - nd:norb - n_buffer_r - 2 * nr]
    maxij3 = 0
    for row in VRD:
        nz = np.nonzero(row)[0]
        if nz.size and nz[0] + 1 >= 2:
            maxij3 = max(maxij3, nd - int(nz[0]))
    HD = A[d0:d0 + nd, d0:d0 + nd]
    # last[r]: last nonzero column (1-based, 0 if none) of HD row r (1-based)
    last = np.zeros(nd + 2, dtype=np.int64)
    for r in range(nd):
        nz = np.nonzero(HD[r])[0]
        last[r + 1] = nz[-1] + 1 if nz.size else 0

    def reach(r0, r1):            # last nonzero column of rows r0..r1 (1-based, inclusive)
        return int(last[r0:r1 + 1].max()) if r1 >= r0 else 0

    def col_any(r0, r1, c):       # any nonzero HD(r0:r1, c)
        return r1 >= r0 and 1 <= c <= nd and bool(HD[r0 - 1:r1, c - 1].any())

    def row_any(r, c0):           # any nonzero HD(r, c0:nd)
        return 1 <= r <= nd and c0 <= nd and bool(HD[r - 1, max(c0, 1) - 1:].any())

    layers = []
    start, cont, start0 = 1, 0, 1
    lay1 = lay2 = None
    while start < nd - 1 and cont < 2 and start >= start0:
        best = 0
        start0 = start
        if cont == 0:
            for i in range(maxij1, nd - 1):
                layer1 = i + 1 - start
                for j in range(i + 1, nd):
                    layer2 = j - i
                    ncol = nd - j
                    if ncol <= best:
                        break           # later j only shrink the far block
                    cl = start + layer1 + layer2 - 1
                    if (col_any(start, start + layer1 - 1, cl) and row_any(start + layer1, cl + 1)
                            and reach(start, start + layer1 - 1) <= cl):
                        best = ncol
                        lay1, lay2 = layer1, layer2
                        layers.append(lay1)
            cont += 1
            if lay1 is None:
                raise ValueError("blockwise_setup: no first layer found")
            start += lay1
        else:
            layer1 = lay2
            cont = 2
            for j in range(start + layer1, nd):
                layer2 = j + 1 - start - layer1
                ncol = nd - j
                if ncol <= best:
                    break
                cl = start + layer1 + layer2 - 1
                if col_any(start, start + layer1 - 1, cl) and reach(start, start + layer1 - 1) <= cl:
                    best = ncol
                    lay1, lay2 = layer1, layer2
                    layers.append(lay1)
                    cont = 1
                    start += lay1
                    if start + layer1 + layer2 == nd + 1:
                        layers.append(lay1)
    layers.append(nd - sum(layers))
    while len(layers) > 1 and layers[-1] < maxij3:
        tail = layers.pop()
        layers[-1] += tail
    return layers


def gen_dyn_host(fc, tables, masses, recivec, kfrac, nbx, nby, n_uc, nz, hermitize=True):
    """D(q) through the reference-layout host entry pf_gen_dyn (the arrays
    as negf/phinfortran.f90 holds them).  Returns (nq, norb, norb) complex."""
    lib = _abi.load()
    fc = np.asarray(fc, dtype=np.float64)
    natoms = tables.num.shape[0]
    norb = 3 * natoms
    fcf = np.asfortranarray(fc)
    num = np.asfortranarray(tables.num.astype(np.int32))
    nent = int(tables.idx.size)
    idx1 = np.ascontiguousarray(tables.idx + 1, dtype=np.int32)
    drf = np.asfortranarray(tables.dr.reshape(-1, 3)) if nent else np.zeros((1, 3), order="F")
    m = np.ascontiguousarray(masses, dtype=np.float64)
    rv = np.ascontiguousarray(recivec, dtype=np.float64)
    k = np.ascontiguousarray(np.atleast_2d(kfrac), dtype=np.float64)
    nq = k.shape[0]
    out = np.zeros((nq, norb, norb), dtype=np.complex128)   # [q][col][row] = column-major per q
    rc = lib.pf_gen_dyn(natoms, nbx, nby, n_uc, nz, fc.shape[0], fc.shape[1], _p(fcf), _p(num, C.c_int), nent,
                        _p(idx1, C.c_int), _p(drf), _p(m), _p(rv), nq, _p(k), int(bool(hermitize)),
                        _p(out.view(np.float64)))
    if rc != 0:
        raise _abi.PFError(rc, lib.pf_fullh_last_error().decode(errors="replace"))
    return np.swapaxes(out, -1, -2)


class FullH:
    """Device-resident set-up of a binary force-constant system.

    fc (3 n_uc, 3 n_sc) eV/A^2; tables from ``fc_tables``; masses per
    structure atom (amu); recivec rows = reciprocal vectors of the structure
    cell; lead sizes nl, nr and buffers n_buffer_l, n_buffer_r in orbitals;
    layer_list from ``blockwise_setup``."""

    def __init__(self, fc, tables, masses, recivec, nbx, nby, n_uc, nz, *, nl, nr, n_buffer_l, n_buffer_r,
                 layer_list, device="cuda"):
        import torch
        self.torch = torch
        fc = np.asarray(fc, dtype=np.float64)
        natoms = tables.num.shape[0]
        self.natoms, self.norb = natoms, 3 * natoms
        self.fc_rows = fc.shape[0]
        pa, pb, off = tables.pairs()
        if tables.idx.size and (tables.idx.min() < 0 or 3 * (tables.idx.max() + 1) > fc.shape[1]):
            raise ValueError("fc column atom out of range")
        rows = row_atoms(natoms, nbx, nby, n_uc, nz)
        if 3 * (rows.max() + 1) > fc.shape[0]:
            raise ValueError("fc row atom out of range")
        t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).to(device)
        self.d_fc = t(np.asfortranarray(fc).ravel(order="F"), np.float64)
        self.d_pa, self.d_pb, self.d_off = t(pa, np.int32), t(pb, np.int32), t(off, np.int32)
        self.npairs = int(pa.size)
        self.d_idx = t(tables.idx if tables.idx.size else np.zeros(1), np.int32)
        self.d_dr = t(tables.dr if tables.dr.size else np.zeros((1, 3)), np.float64)
        self.d_row = t(rows, np.int32)
        self.d_mass = t(masses, np.float64)
        self.recivec = np.asarray(recivec, dtype=np.float64)
        self.nl, self.nr, self.nbl, self.nbr = nl, nr, n_buffer_l, n_buffer_r
        self.layer_list = [int(x) for x in layer_list]
        if sum(self.layer_list) != self.norb - n_buffer_l - n_buffer_r - 2 * nl - 2 * nr:
            raise ValueError("layer_list does not cover the device")
        self.n = max(self.layer_list)
        self.d_ls = t(np.concatenate([[0], np.cumsum(self.layer_list)]), np.int32)
        self.device = device

    def dynamical(self, kfrac, hermitize=True, stream=None):
        """(nq, norb, norb) complex128 device tensor of D(q) in the C ABI
        layout (element [q, c, r] = D(r, c); ``.transpose(-1, -2)`` gives the
        matrix)."""
        torch = self.torch
        lib = _abi.load()
        k = np.atleast_2d(np.asarray(kfrac, dtype=np.float64)) @ self.recivec
        nq = k.shape[0]
        kd = torch.from_numpy(np.ascontiguousarray(k)).to(self.device)
        H = torch.empty((nq, self.norb, self.norb), dtype=torch.complex128, device=self.device)
        s = stream if stream is not None else torch.cuda.current_stream()
        rc = lib.pf_gen_dyn_dev(self.natoms, self.fc_rows, self.d_fc.data_ptr(), self.npairs, self.d_pa.data_ptr(),
                                self.d_pb.data_ptr(), self.d_off.data_ptr(), self.d_idx.data_ptr(),
                                self.d_dr.data_ptr(), self.d_row.data_ptr(), self.d_mass.data_ptr(), nq,
                                kd.data_ptr(), int(bool(hermitize)), H.data_ptr(), C.c_void_p(s.cuda_stream))
        if rc != 0:
            raise _abi.PFError(rc, lib.pf_fullh_last_error().decode(errors="replace"))
        return H

    def blocks(self, H, stream=None):
        """Device block set (C ABI layout) sliced from the dense matrices H
        (as returned by ``dynamical``); returns (dev dict, dims)."""
        torch = self.torch
        lib = _abi.load()
        nq = H.shape[0]
        n, nl, nr, L = self.n, self.nl, self.nr, len(self.layer_list)
        shapes = {"HL": (nl, nl), "HLv": (nl, nl), "HR": (nr, nr), "HRv": (nr, nr), "Hd": (L, n, n),
                  "Hdv": (max(L - 1, 0), n, n), "Hld": (n, nl), "Hrd": (n, nr)}
        dev = {k: torch.zeros((nq,) + v + (2,), dtype=torch.float64, device=self.device) for k, v in shapes.items()}
        bad = torch.zeros(1, dtype=torch.int32, device=self.device)
        s = stream if stream is not None else torch.cuda.current_stream()
        rc = lib.pf_dense_to_tdb_dev(self.norb, nq, H.data_ptr(), nl, nr, self.nbl, self.nbr, L, self.d_ls.data_ptr(),
                                     n, *[dev[k].data_ptr() for k in BLOCK_NAMES], bad.data_ptr(),
                                     C.c_void_p(s.cuda_stream))
        if rc != 0:
            raise _abi.PFError(rc, lib.pf_fullh_last_error().decode(errors="replace"))
        if int(bad.item()) != 0:
            raise _abi.PFError(-1, "pf_dense_to_tdb: a slice leaves the matrix")
        return dev, (n, nl, nr, L, nq)

    def transport(self, E, kfrac, qidx=None, *, eta, eta0, convergence, dev_factor=10.0, max_iter=1000,
                  precision="fp64", refine_iters=2, want_transr=False):
        """T_L of every point (E[p] at k = kfrac[qidx[p]]): D(q) built and
        sliced on the GPU, then the tdb transport engine on device blocks.
        want_transr (FP64 and the large-block arithmetics) adds T_R from the
        right-to-left sweep of G_block (negf/device.f90:289-560) as transr,
        without the reference's debug override of G_NN near E = 31.2954
        (device.f90:485-493)."""
        if want_transr and precision == "mixed":
            raise ValueError("the mixed path computes T_L only")
        from .transport import DeviceTransport
        torch = self.torch
        H = self.dynamical(kfrac)
        dev, dims = self.blocks(H)
        E = np.ascontiguousarray(E, dtype=np.float64)
        if max(dims[0], dims[1], dims[2]) > 48:
            # layers above the resident size: the tiled engine through the host entry
            from .transport import transport_tdb
            blocks = {k: np.swapaxes(v[..., 0].cpu().numpy() + 1j * v[..., 1].cpu().numpy(), -1, -2)
                      for k, v in dev.items()}
            return transport_tdb(E, blocks, eta=eta, eta0=eta0, convergence=convergence, dev_factor=dev_factor,
                                 qidx=qidx, max_iter=max_iter, want_transr=want_transr, check=False,
                                 precision=precision)
        tr = DeviceTransport.from_device({k: v.reshape(-1) for k, v in dev.items()}, dims, E.size, eta=eta,
                                         eta0=eta0, convergence=convergence, dev_factor=dev_factor,
                                         max_iter=max_iter, precision=precision, refine_iters=refine_iters,
                                         device=self.device, want_transr=want_transr)
        Ed = torch.from_numpy(E).to(self.device)
        qd = None if qidx is None else torch.from_numpy(np.ascontiguousarray(qidx, dtype=np.int32)).to(self.device)
        tl, trr, st = tr.run(Ed, qd)
        torch.cuda.synchronize()
        out = dict(transl=tl.cpu().numpy().copy(), status=st.cpu().numpy().copy())
        if want_transr:
            out["transr"] = trr.cpu().numpy().copy()
        return out
