"""Restatement of the binary force-constant (full-Hamiltonian) phonon path
(oracle; tests only).

* ``read_binary_fc``      -- negf/fc.f90:25-44 (raw real(8) stream, column-major)
* ``fc_sc_positions``     -- negf/input.f90:442-473 (fc supercell positions)
* ``asr_cutoff``          -- negf/dyn.f90:1218-1271 (zero pairs beyond r_cut,
                             acoustic sum rule on the self term)
* ``fc_to_dyn_idx``       -- negf/dyn.f90:988-1093 (gen_fc_to_dyn_idx) plus the
                             row-major flattening of negf/phinfortran.f90:655-683
* ``lead_fc_to_dyn_idx``  -- negf/dyn.f90:1095-1216 (gen_lead_fc_to_dyn_idx)
* ``gen_dyn``             -- negf/dyn.f90:39-150 (dense norb x norb D(q))
* ``gen_dyn_lead``        -- negf/dyn.f90:190-312 (lead D(q) and its coupling)
* ``swap_lead_region``    -- negf/dyn.f90:917-986
* ``blockwise_setup``     -- negf/device.f90:11-249 (layer partition of the device)
* ``dense_to_tdb``        -- the slices negf/surface.f90:170-198 and
                             negf/device.f90:323-500 take from the dense matrix,
                             as the block set of the tdb transport path

Indices are 0-based here; a comment gives the reference's 1-based form
where the arithmetic differs.  Positions are in Angstrom, force constants
in eV/A^2, masses in amu, D(q) in THz^2 (negf/dyn.f90:138).
"""
from __future__ import annotations

import numpy as np

PI = 3.141592653589793238          # negf/util.f90:5
ELE_VOLT = 1.609e-19                # negf/util.f90:7 (sic)
MASS_PROTON = 1.6726219e-27         # negf/util.f90:8
BLOCK_TOL = 1.0e-7                  # negf/device.f90:43-131 sparsity threshold


def to_thz2(h):
    """negf/dyn.f90:138: Ham*eleVolt/1.0d-20/mass_proton/(1.0d12*2.0d0*pi)**2,
    evaluated left to right."""
    return h * ELE_VOLT / 1.0e-20 / MASS_PROTON / (1.0e12 * 2.0 * PI) ** 2


def hermitian(a):
    """negf/util.f90:940-949: 0.5 (A + A^H)."""
    return 0.5 * (a + a.conj().T)


def read_binary_fc(path, nr, nc):
    """negf/fc.f90:25-44: nr x nc real(8) values, Fortran (column-major) order."""
    d = np.fromfile(path, dtype="<f8", count=nr * nc)
    if d.size != nr * nc:
        raise ValueError("short force-constant file")
    return d.reshape(nc, nr).T.copy()


def fc_sc_positions(pos, nx, ny, nz, cell):
    """negf/input.f90:442-473.  pos (natoms, 4) -> (natoms*(2nx+1)(2ny+1)(2nz+1), 4);
    supercell atom ((i+nx)(2ny+1)(2nz+1) + (j+ny)(2nz+1) + nz + k) * natoms + n."""
    pos = np.asarray(pos, dtype=np.float64)
    cell = np.asarray(cell, dtype=np.float64)
    na = pos.shape[0]
    out = np.zeros((na * (2 * nx + 1) * (2 * ny + 1) * (2 * nz + 1), 4))
    for i in range(-nx, nx + 1):
        for j in range(-ny, ny + 1):
            for k in range(-nz, nz + 1):
                base = ((i + nx) * (2 * ny + 1) * (2 * nz + 1) + (j + ny) * (2 * nz + 1) + nz + k) * na
                shift = np.array([float(i), float(j), float(k)]) @ cell
                out[base:base + na, 0:3] = pos[:, 0:3] + shift
                out[base:base + na, 3] = pos[:, 3]
    return out


def central_start(n_uc, nx, ny, nz):
    """0-based first fc column atom of the central cell (negf/dyn.f90:1243-1244,
    istart - 1)."""
    return n_uc * (nx * (2 * ny + 1) * (2 * nz + 1) + ny * (2 * nz + 1) + nz)


def asr_cutoff(fc, pos, rcut, nx, ny, nz):
    """negf/dyn.f90:1218-1271.  fc (3m, 3n), pos = the fc supercell positions."""
    fc = np.array(fc, dtype=np.float64)
    m = fc.shape[0] // 3
    n = fc.shape[1] // 3
    i0 = central_start(m, nx, ny, nz)
    new = fc.copy()
    for i in range(m):
        for j in range(n):
            dr = pos[j, 0:3] - pos[i + i0, 0:3]
            if np.sqrt(np.dot(dr, dr)) > rcut:
                new[3 * i:3 * i + 3, 3 * j:3 * j + 3] = 0.0
    for i in range(m):
        for ic in range(3):
            for jc in range(3):
                row = 3 * i + ic
                self_col = 3 * (i + i0) + jc
                tot = 0.0
                for v in new[row, jc:3 * n:3]:
                    tot += v
                new[row, self_col] = -(tot - new[row, self_col])
    return new


def _matches(pos_sc, i_fc, dr, cells):
    """fc atoms idx (ascending) of the listed supercell cells with
    |pos_sc[idx] - pos_sc[i_fc] - dr| < 1e-3 (negf/dyn.f90:1072-1081)."""
    out = []
    for i_uc, n_uc in cells:
        idx = np.arange(i_uc * n_uc, (i_uc + 1) * n_uc)
        d = pos_sc[idx, 0:3] - pos_sc[i_fc, 0:3] - dr
        hit = np.sqrt(np.einsum("ij,ij->i", d, d)) < 1.0e-3
        out.extend(int(v) for v in idx[hit])
    return out


def fc_to_dyn_idx(pos_sc, pos_s, cell, nbx, nby, n_uc, nz, nfc, r_cutoff):
    """negf/dyn.f90:988-1093 and the flattening of negf/phinfortran.f90:665-683.

    Returns (num, idx, dr): num[a, b] entries for the atom pair (a, b); the
    entries of all pairs in row-major (a, b) order, each the 0-based fc
    column atom idx and the bond vector dr."""
    nx, ny, nzf = nfc
    pos_sc = np.asarray(pos_sc, dtype=np.float64)
    pos_s = np.asarray(pos_s, dtype=np.float64)
    cell = np.asarray(cell, dtype=np.float64)
    natoms = pos_s.shape[0]
    i0 = central_start(n_uc, nx, ny, nzf)
    per = n_uc // nz
    cells = [(((ii * (2 * ny + 1) * (2 * nzf + 1)) + jj * (2 * nzf + 1) + kk), n_uc)
             for ii in range(2 * nx + 1) for jj in range(2 * ny + 1) for kk in range(2 * nzf + 1)]
    num = np.zeros((natoms, natoms), dtype=np.int64)
    lists = {}
    for iy in range(nby):
        for ix in range(nbx):
            for iz in range(nz):
                for is_ in range(per):
                    i = i0 + iz * per + is_
                    a = iz * nby * nbx * per + iy * nbx * per + ix * per + is_
                    for b in range(natoms):
                        ent = []
                        for dx in (-1, 0, 1):
                            for dy in (-1, 0, 1):
                                for dz in (-1, 0, 1):
                                    shift = np.array([float(dx), float(dy), float(dz)]) @ cell
                                    dr = pos_s[b, 0:3] + shift - pos_s[a, 0:3]
                                    if np.sqrt(np.dot(dr, dr)) < r_cutoff:
                                        for idx in _matches(pos_sc, i, dr, cells):
                                            ent.append((idx, dr.copy()))
                        num[a, b] = len(ent)
                        if ent:
                            lists[(a, b)] = ent
    idx, drs = [], []
    for a in range(natoms):
        for b in range(natoms):
            for e in lists.get((a, b), ()):
                idx.append(e[0])
                drs.append(e[1])
    return num, np.array(idx, dtype=np.int64), np.array(drs, dtype=np.float64).reshape(-1, 3)


def lead_fc_to_dyn_idx(pos_sc, pos_s, cell, nbx, nby, n_uc, nfc, r_cutoff):
    """negf/dyn.f90:1095-1216: the same for a lead principal layer; the
    in-layer entries take fc cells with kk = n_fc_uc_z (the central z cell),
    the coupling entries cells with kk = 2 n_fc_uc_z (1-based 2 nz + 1).
    Returns (num, idx, dr, num_v, idx_v, dr_v)."""
    nx, ny, nzf = nfc
    pos_sc = np.asarray(pos_sc, dtype=np.float64)
    pos_s = np.asarray(pos_s, dtype=np.float64)
    cell = np.asarray(cell, dtype=np.float64)
    natoms = pos_s.shape[0]
    i0 = central_start(n_uc, nx, ny, nzf)
    num = np.zeros((natoms, natoms), dtype=np.int64)
    num_v = np.zeros((natoms, natoms), dtype=np.int64)
    lists, lists_v = {}, {}
    for iy in range(nby):
        for ix in range(nbx):
            for is_ in range(n_uc):
                i = i0 + is_
                a = iy * nbx * n_uc + ix * n_uc + is_
                for b in range(natoms):
                    ent, ent_v = [], []
                    for dx in (-1, 0, 1):
                        for dy in (-1, 0, 1):
                            for dz in (-1, 0, 1):
                                shift = np.array([float(dx), float(dy), float(dz)]) @ cell
                                dr = pos_s[b, 0:3] + shift - pos_s[a, 0:3]
                                if np.sqrt(np.dot(dr, dr)) < r_cutoff:
                                    for ii in range(2 * nx + 1):
                                        for jj in range(2 * ny + 1):
                                            c0 = ii * (2 * ny + 1) * (2 * nzf + 1) + jj * (2 * nzf + 1)
                                            for idx in _matches(pos_sc, i, dr, [(c0 + nzf, n_uc)]):
                                                ent.append((idx, dr.copy()))
                                            for idx in _matches(pos_sc, i, dr, [(c0 + 2 * nzf, n_uc)]):
                                                ent_v.append((idx, dr.copy()))
                    num[a, b] = len(ent)
                    num_v[a, b] = len(ent_v)
                    if ent:
                        lists[(a, b)] = ent
                    if ent_v:
                        lists_v[(a, b)] = ent_v

    def flat(L):
        idx, drs = [], []
        for a in range(natoms):
            for b in range(natoms):
                for e in L.get((a, b), ()):
                    idx.append(e[0])
                    drs.append(e[1])
        return np.array(idx, dtype=np.int64), np.array(drs, dtype=np.float64).reshape(-1, 3)

    idx, dr = flat(lists)
    idx_v, dr_v = flat(lists_v)
    return num, idx, dr, num_v, idx_v, dr_v


def _accumulate(H, a, b, row_atom, m1, m2, fc, idx, dr, t, n, kc):
    """Add the n entries starting at t of the pair (a, b) (negf/dyn.f90:110-130)."""
    for _ in range(n):
        d = dr[t]
        j = idx[t]
        t += 1
        ph = np.exp(1j * np.dot(d, kc))
        for ic in range(3):
            for jc in range(3):
                H[3 * a + ic, 3 * b + jc] += fc[3 * row_atom + ic, 3 * j + jc] * ph / np.sqrt(m1 * m2)
    return t


def gen_dyn(kpoint, fc, masses, recivec, num, idx, dr, nbx, nby, n_uc, nz):
    """negf/dyn.f90:39-150: dense D(q) (norb x norb, THz^2), Hermitised.
    kpoint is fractional (kpoint_cart = kpoint . recivec); masses per atom."""
    natoms = num.shape[0]
    H = np.zeros((3 * natoms, 3 * natoms), dtype=np.complex128)
    kc = np.asarray(kpoint, dtype=np.float64) @ np.asarray(recivec, dtype=np.float64)
    per = n_uc // nz
    t = 0
    for a in range(natoms):
        iz = a // (nby * nbx * per)
        rem = a - iz * nby * nbx * per
        iy = rem // (nbx * per)
        rem -= iy * nbx * per
        ix = rem // per
        is_ = rem - ix * per
        row_atom = iz * per + is_
        for b in range(natoms):
            if num[a, b] > 0:
                t = _accumulate(H, a, b, row_atom, masses[a], masses[b], fc, idx, dr, t, num[a, b], kc)
    return hermitian(to_thz2(H))


def gen_dyn_lead(kpoint, fc, masses, recivec, num, idx, dr, num_v, idx_v, dr_v, nbx, nby, n_uc):
    """negf/dyn.f90:190-312: lead layer D(q) (Hermitised) and its coupling to
    the next layer (not Hermitised), both THz^2."""
    natoms = num.shape[0]
    H = np.zeros((3 * natoms, 3 * natoms), dtype=np.complex128)
    Hv = np.zeros_like(H)
    kc = np.asarray(kpoint, dtype=np.float64) @ np.asarray(recivec, dtype=np.float64)
    t = tv = 0
    for a in range(natoms):
        iy = a // (nbx * n_uc)
        rem = a - iy * nbx * n_uc
        ix = rem // n_uc
        row_atom = rem - ix * n_uc
        for b in range(natoms):
            if num[a, b] > 0:
                t = _accumulate(H, a, b, row_atom, masses[a], masses[b], fc, idx, dr, t, num[a, b], kc)
            if num_v[a, b] > 0:
                tv = _accumulate(Hv, a, b, row_atom, masses[a], masses[b], fc, idx_v, dr_v, tv, num_v[a, b], kc)
    return hermitian(to_thz2(H)), to_thz2(Hv)


def swap_lead_region(H, Hl, Hr, Hlv, Hrv, natoms, buffer_left, period_left, buffer_right, period_right):
    """negf/dyn.f90:917-986 (atoms counts; 0-based half-open slices)."""
    H = np.array(H, dtype=np.complex128)
    pl, pr = 3 * period_left, 3 * period_right
    lefta = 3 * buffer_left
    rightc = 3 * natoms - 3 * buffer_right
    for i in (1, 2):
        H[lefta + (i - 1) * pl:lefta + i * pl, lefta + (i - 1) * pl:lefta + i * pl] = Hl
        H[rightc - i * pr:rightc - (i - 1) * pr, rightc - i * pr:rightc - (i - 1) * pr] = Hr
    leftb = lefta + pl
    leftc = lefta + 2 * pl
    H[lefta:leftb, leftb:leftc] = Hlv
    H[leftb:leftc, lefta:leftb] = Hlv.conj().T
    righta = rightc - 2 * pr
    rightb = rightc - pr
    H[righta:rightb, rightb:rightc] = Hrv
    H[rightb:rightc, righta:rightb] = Hrv.conj().T
    return hermitian(H)


def blockwise_setup(H, nl, nr, n_buffer_l, n_buffer_r):
    """negf/device.f90:11-249: partition the device part of the dense matrix
    into layers.  Returns layer_list (orbital counts).  The scan keeps the
    reference's 1-based loop variables; HD(r, c) below is 1-based."""
    H = np.asarray(H)
    norb = H.shape[0]
    tol = BLOCK_TOL
    nd = norb - n_buffer_l - n_buffer_r - 2 * nl - 2 * nr
    d0 = n_buffer_l + 2 * nl
    A = np.abs(H)
    VLD = A[n_buffer_l + nl:n_buffer_l + 2 * nl, d0:d0 + nd]
    maxij1 = 0
    for i in range(1, nl + 1):
        for j in range(1, nd):
            if VLD[i - 1, j - 1] > tol and np.max(VLD[i - 1, j:nd]) < tol and j >= maxij1:
                maxij1 = j
    VRD = A[norb - n_buffer_r - 2 * nr:norb - n_buffer_r - nr, norb - n_buffer_r - 2 * nr - nd:norb - n_buffer_r - 2 * nr]
    maxij3 = 0
    for i in range(1, nr + 1):
        for j in range(2, nd + 1):
            if VRD[i - 1, j - 1] > tol and np.max(VRD[i - 1, 0:j - 1]) < tol and nd - j + 1 > maxij3:
                maxij3 = nd - j + 1
    HD = A[d0:d0 + nd, d0:d0 + nd]

    def hd(r0, r1, c0, c1):          # HD(r0:r1, c0:c1), 1-based inclusive
        return HD[r0 - 1:r1, c0 - 1:c1]

    def mx(x):                       # Fortran maxval of an empty array is -huge
        return np.max(x) if x.size else -np.inf

    layers = []                      # layer_list entries appended so far
    start, cont, start0 = 1, 0, 1
    lay1 = lay2 = None
    while start < nd - 1 and cont < 2 and start >= start0:
        maxij2 = 0
        start0 = start
        if cont == 0:
            for i in range(maxij1, nd - 1):
                for j in range(i + 1, nd):
                    layer1 = i + 1 - start
                    layer2 = j - i
                    ncol = nd - start - layer1 - layer2 + 1
                    vt = hd(start, start + layer1 - 1, start + layer1 + layer2, nd)
                    vl = hd(start, start + layer1 - 1, start + layer1 + layer2 - 1, start + layer1 + layer2 - 1)
                    vb = hd(start + layer1, start + layer1, start + layer1 + layer2, nd)
                    if mx(vl) > tol and mx(vb) > tol and mx(vt) < tol and ncol > maxij2:
                        maxij2 = ncol
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
                ncol = nd - start - layer1 - layer2 + 1
                vt = hd(start, start + layer1 - 1, start + layer1 + layer2, nd)
                vl = hd(start, start + layer1 - 1, start + layer1 + layer2 - 1, start + layer1 + layer2 - 1)
                if mx(vl) > tol and mx(vt) < tol and ncol > maxij2:
                    maxij2 = ncol
                    lay1, lay2 = layer1, layer2
                    layers.append(lay1)
                    cont = 1
                    start += lay1
                    if start + layer1 + layer2 == nd + 1:
                        layers.append(lay1)
    layers.append(nd - sum(layers))
    while len(layers) > 1 and layers[-1] < maxij3:
        last = layers.pop()
        layers[-1] += last
    return layers


def dense_to_tdb(H, layer_list, nl, nr, n_buffer_l, n_buffer_r, n=None):
    """The block set of the tdb path taken from the dense matrix as
    negf/surface.f90:170-198 (lead cells) and negf/device.f90:323-500 (device
    layers and couplings) slice it; every device layer is zero-padded to n
    (default max(layer_list)).  The padding decouples: its rows and columns
    of every coupling are zero, so T is unchanged."""
    H = np.asarray(H, dtype=np.complex128)
    norb = H.shape[0]
    L = len(layer_list)
    n = int(n or max(layer_list))
    d0 = n_buffer_l + 2 * nl
    starts = np.concatenate([[0], np.cumsum(layer_list)]).astype(int) + d0
    ol = slice(n_buffer_l + nl, n_buffer_l + 2 * nl)       # left cell next to the device
    il = slice(n_buffer_l, n_buffer_l + nl)                # outer left cell
    orr = slice(norb - n_buffer_r - 2 * nr, norb - n_buffer_r - nr)
    ir = slice(norb - n_buffer_r - nr, norb - n_buffer_r)
    Hd = np.zeros((L, n, n), dtype=np.complex128)
    Hdv = np.zeros((max(L - 1, 0), n, n), dtype=np.complex128)
    for j in range(L):
        s = slice(starts[j], starts[j + 1])
        dj = layer_list[j]
        Hd[j, :dj, :dj] = H[s, s]
        if j + 1 < L:
            s2 = slice(starts[j + 1], starts[j + 2])
            Hdv[j, :dj, :layer_list[j + 1]] = H[s, s2]
    Hld = np.zeros((nl, n), dtype=np.complex128)
    Hld[:, :layer_list[0]] = H[ol, starts[0]:starts[1]]
    Hrd = np.zeros((nr, n), dtype=np.complex128)
    Hrd[:, :layer_list[-1]] = H[orr, starts[L - 1]:starts[L]]
    return dict(HL=H[ol, ol].copy(), HLv=H[il, ol].copy(), HR=H[orr, orr].copy(), HRv=H[ir, orr].copy(),
                Hd=Hd, Hdv=Hdv, Hld=Hld, Hrd=Hrd)
