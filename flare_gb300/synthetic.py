"""Seeded synthetic structures and Lennard-Jones labels.

The workloads are described by what they are:
  * ``fcc_al``      FCC Al-like supercell (a = 4.05 A), Gaussian displacements;
  * ``random_alloy`` random sequential addition at a given density with a
                    periodic minimum distance, species drawn from fractions.
Labels come from a truncated Lennard-Jones pair potential with Lorentz-
Berthelot mixing (eps_ab = sqrt(eps_a eps_b), sigma_ab = (sigma_a+sigma_b)/2),
standing in for the ASE LennardJones calculator used by the reference's test
fixtures (tests/get_sgp.py:7,127), which is not installed here.

All random numbers come from ``numpy.random.Generator(PCG64(seed))``.
"""
import numpy as np


def rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def fcc_al(n_cells=4, a=4.05, sigma=0.05, seed=0):
    """n_cells^3 conventional FCC cells (4 atoms each), cubic, periodic."""
    basis = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]])
    g = np.stack(np.meshgrid(*[np.arange(n_cells)] * 3, indexing="ij"),
                 -1).reshape(-1, 3)
    pos = ((g[:, None, :] + basis[None]) * a).reshape(-1, 3)
    cell = np.eye(3) * (a * n_cells)
    pos = pos + rng(seed).normal(scale=sigma, size=pos.shape)
    return cell, np.zeros(len(pos), dtype=np.int64), pos


def random_alloy(n_atoms, density=0.06, fractions=(0.5, 0.5), dmin=1.8,
                 seed=0):
    """Cubic cell at ``density`` atoms/A^3; positions by random sequential
    addition with a periodic minimum distance ``dmin``; species i.i.d. from
    ``fractions``."""
    r = rng(seed)
    L = (n_atoms / density) ** (1.0 / 3.0)
    pos = np.zeros((n_atoms, 3))
    k = 0
    tries = 0
    while k < n_atoms:
        cand = r.uniform(0, L, size=3)
        d = pos[:k] - cand
        d -= L * np.round(d / L)
        if k == 0 or np.min(np.einsum("ij,ij->i", d, d)) >= dmin * dmin:
            pos[k] = cand
            k += 1
        tries += 1
        if tries > 200 * n_atoms:
            raise RuntimeError("random sequential addition did not converge")
    fr = np.asarray(fractions, dtype=np.float64)
    species = r.choice(len(fr), size=n_atoms, p=fr / fr.sum())
    return np.eye(3) * L, species.astype(np.int64), pos


def rsa_alloy(n_atoms, density=0.06, fractions=(0.5, 0.5), dmin=1.8, seed=0,
              batch=256):
    """Cubic cell at ``density`` atoms/A^3 filled by random sequential
    addition with a periodic minimum distance ``dmin``, species i.i.d. from
    ``fractions`` — the same process as ``random_alloy``, with candidates
    proposed in batches and tested against a grid of dmin-wide cells, so a
    2000-atom cell takes milliseconds (its random stream differs from
    ``random_alloy``'s)."""
    r = rng(seed)
    L = (n_atoms / density) ** (1.0 / 3.0)
    nc = max(1, int(np.floor(L / dmin)))
    cap = 8                                   # points >= dmin apart per cell
    grid = np.full((nc, nc, nc, cap), -1, dtype=np.int64)
    fill = np.zeros((nc, nc, nc), dtype=np.int64)
    pos = np.zeros((n_atoms, 3))
    d2min = dmin * dmin
    offs = np.array([(a, b, c) for a in (-1, 0, 1) for b in (-1, 0, 1)
                     for c in (-1, 0, 1)]) if nc >= 3 else None
    k = 0
    tries = 0
    while k < n_atoms:
        cand = r.uniform(0, L, size=(batch, 3))
        tries += batch
        if tries > 200 * n_atoms + batch:
            raise RuntimeError("random sequential addition did not converge")
        cell = np.minimum((cand / L * nc).astype(np.int64), nc - 1)
        if offs is not None:
            nb = (cell[:, None, :] + offs[None, :, :]) % nc     # B x 27 x 3
            idx = grid[nb[..., 0], nb[..., 1], nb[..., 2]].reshape(batch, -1)
        else:
            idx = np.broadcast_to(np.arange(k), (batch, k))
        ok = np.ones(batch, dtype=bool)
        if idx.shape[1]:
            valid = idx >= 0
            d = pos[np.where(valid, idx, 0)] - cand[:, None, :]
            d -= L * np.round(d / L)
            r2 = np.einsum("bkx,bkx->bk", d, d)
            ok = ~np.any(valid & (r2 < d2min), axis=1)
        # accept in order; a candidate conflicting with an earlier accepted
        # one of the same batch is rejected (conflicts are rare: only those
        # columns are walked)
        okidx = np.nonzero(ok)[0]
        cb = cand[okidx]
        d = cb[:, None, :] - cb[None, :, :]
        d -= L * np.round(d / L)
        conflict = np.triu(np.einsum("ijx,ijx->ij", d, d) < d2min, 1)
        keep = np.ones(len(okidx), dtype=bool)
        for j in np.nonzero(conflict.any(axis=0))[0]:
            if np.any(conflict[:j, j] & keep[:j]):
                keep[j] = False
        acc = okidx[keep][:n_atoms - k]
        for b in acc:
            pos[k] = cand[b]
            i, j, l = cell[b]
            if fill[i, j, l] >= cap:
                raise RuntimeError("grid cell overflow")
            grid[i, j, l, fill[i, j, l]] = k
            fill[i, j, l] += 1
            k += 1
    fr = np.asarray(fractions, dtype=np.float64)
    species = r.choice(len(fr), size=n_atoms, p=fr / fr.sum())
    return np.eye(3) * L, species.astype(np.int64), pos


def _pairs(cell, pos, rc):
    """All (i, j, image) pairs with 0 < |r_ij| < rc, by a sweep over the
    images needed for this cell.  Returns i, j, r_ij vectors."""
    inv = np.linalg.inv(cell)
    h = 1.0 / np.linalg.norm(inv, axis=0)          # plane spacings
    nimg = np.ceil(rc / h).astype(int)
    frac = pos @ inv
    frac -= np.floor(frac)
    w = frac @ cell
    shifts = np.stack(np.meshgrid(*[np.arange(-k, k + 1) for k in nimg],
                                  indexing="ij"), -1).reshape(-1, 3)
    I, J, V = [], [], []
    for s in shifts:
        off = s @ cell
        d = w[None, :, :] - w[:, None, :] + off
        r2 = np.einsum("ijk,ijk->ij", d, d)
        m = (r2 < rc * rc) & (r2 > 0)
        ii, jj = np.nonzero(m)
        I.append(ii)
        J.append(jj)
        V.append(d[ii, jj])
    return np.concatenate(I), np.concatenate(J), np.concatenate(V)


def lennard_jones(cell, species, pos, eps, sig, rc):
    """Truncated LJ energy (eV), forces (eV/A) and stress (eV/A^3, flare
    order xx, xy, xz, yy, yz, zz; sign convention of the SGP kernel's stress
    columns, sigma_ab = -(1/V) sum_pairs dE/dr_ij,a r_ij,b)."""
    eps = np.asarray(eps, dtype=np.float64)
    sig = np.asarray(sig, dtype=np.float64)
    sp = np.asarray(species)
    i, j, v = _pairs(np.asarray(cell, np.float64), np.asarray(pos, np.float64),
                     rc)
    e_ab = np.sqrt(eps[sp[i]] * eps[sp[j]])
    s_ab = 0.5 * (sig[sp[i]] + sig[sp[j]])
    r = np.linalg.norm(v, axis=1)
    sr6 = (s_ab / r) ** 6
    phi = 4 * e_ab * (sr6 * sr6 - sr6)
    dphi = 4 * e_ab * (-12 * sr6 * sr6 + 6 * sr6) / r
    energy = 0.5 * phi.sum()
    g = (dphi / r)[:, None] * v            # d(phi)/d(r_ij) vector
    forces = np.zeros_like(np.asarray(pos, np.float64))
    np.add.at(forces, i, g)               # F_i = sum_j phi'(r) r_ij / r
    vol = abs(np.linalg.det(cell))
    full = -0.5 * np.einsum("pa,pb->ab", g, v) / vol
    stress = np.array([full[0, 0], full[0, 1], full[0, 2], full[1, 1],
                       full[1, 2], full[2, 2]])
    return energy, forces, stress
