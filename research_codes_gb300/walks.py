"""Host-side i-group / j-list construction for small systems, and the
copyFromFP packers that fill the reference's EPI/EPJ structs.

FDPS builds these lists in the reference (TreeForForceShort::Gather for the
density, ::Symmetry for the hydro force, TreeForForce<SEARCH_MODE_LONG> for
gravity; main.cpp:377-397, calls at hdr_density.hpp:389-397, main.cpp:339-346,
hdr_gravity.hpp:393-402).  FDPS is not part of the reference tree, so list
contents follow this module's own definitions:

  * i-groups: runs of at most `n_group` particles in Morton order;
  * gather (density) list of a group: every particle j with
    dist(x_j, bbox_group) <= max_{i in group} rs_i;
  * symmetric (hydro) list: every j with
    dist(x_j, bbox_group) <= max(max_i h_i, h_j);
  * gravity list: particles within an opening distance of the group as EPJ,
    the remaining particles binned into cells whose monopoles are the SPJ.

The GPU tree builder of the engine produces lists by the same rules at scale;
this module serves the functor-level tests and small demonstrations.
"""
import numpy as np

from . import abi, units


def morton_keys(pos, bits=21):
    lo = pos.min(0)
    span = max(float((pos.max(0) - lo).max()), 1e-300)
    q = np.clip(((pos - lo) / span * ((1 << bits) - 1)).astype(np.uint64), 0, (1 << bits) - 1)

    def spread(v):
        v = v & np.uint64(0x1FFFFF)
        v = (v | (v << np.uint64(32))) & np.uint64(0x1F00000000FFFF)
        v = (v | (v << np.uint64(16))) & np.uint64(0x1F0000FF0000FF)
        v = (v | (v << np.uint64(8))) & np.uint64(0x100F00F00F00F00F)
        v = (v | (v << np.uint64(4))) & np.uint64(0x10C30C30C30C30C3)
        v = (v | (v << np.uint64(2))) & np.uint64(0x1249249249249249)
        return v

    return (spread(q[:, 0]) << np.uint64(2)) | (spread(q[:, 1]) << np.uint64(1)) | spread(q[:, 2])


def make_groups(pos, n_group):
    """Morton-order runs of at most n_group particles: list of index arrays."""
    order = np.argsort(morton_keys(pos), kind="stable")
    return [order[k:k + n_group] for k in range(0, len(order), n_group)]


def _box_dist2(pos, lo, hi):
    d = np.maximum(lo - pos, 0.0) + np.maximum(pos - hi, 0.0)
    return (d * d).sum(1)


def gather_lists(pos, rs, groups):
    out = []
    for g in groups:
        lo, hi = pos[g].min(0), pos[g].max(0)
        r = rs[g].max()
        out.append(np.nonzero(_box_dist2(pos, lo, hi) <= r * r)[0])
    return out


def symmetric_lists(pos, h, groups):
    out = []
    for g in groups:
        lo, hi = pos[g].min(0), pos[g].max(0)
        r = np.maximum(h[g].max(), h)
        out.append(np.nonzero(_box_dist2(pos, lo, hi) <= r * r)[0])
    return out


def gravity_lists(pos, mass, eps2, groups, near_factor=2.0, cell_frac=0.125):
    """EPJ = particles near the group (within near_factor x group size), SPJ =
    monopoles (mass, centre of mass, mass-weighted eps2 as
    hdr_gravity.hpp:37-49) of grid cells over the remaining particles."""
    span = float((pos.max(0) - pos.min(0)).max())
    cell = span * cell_frac
    lo_all = pos.min(0)
    cid = np.floor((pos - lo_all) / cell).astype(np.int64)
    key = (cid[:, 0] * 4096 + cid[:, 1]) * 4096 + cid[:, 2]
    eps, spjs = [], []
    for g in groups:
        lo, hi = pos[g].min(0), pos[g].max(0)
        size = max(float((hi - lo).max()), cell)
        near = _box_dist2(pos, lo, hi) <= (near_factor * size) ** 2
        eps.append(np.nonzero(near)[0])
        far = np.nonzero(~near)[0]
        if len(far):
            uk, inv = np.unique(key[far], return_inverse=True)
            m = np.bincount(inv, weights=mass[far])
            com = np.stack([np.bincount(inv, weights=mass[far] * pos[far, k]) for k in range(3)], 1)
            e2 = np.bincount(inv, weights=mass[far] * eps2[far])
            spj = np.zeros(len(uk), abi.GravitySPJ)
            spj["mass"] = m
            spj["pos"] = com / m[:, None]
            spj["eps2"] = e2 / m
            spjs.append(spj)
        else:
            spjs.append(np.zeros(0, abi.GravitySPJ))
    return eps, spjs


# ---- copyFromFP packers --------------------------------------------------------

def density_epi(idx, s, rs=None):
    """DensityEPI::copyFromFP (hdr_density.hpp:41-48)."""
    a = np.zeros(len(idx), abi.DensityEPI)
    a["id"] = s["id"][idx]
    a["mass"] = s["mass"][idx]
    a["pos"] = s["pos"][idx]
    a["vel"] = s["vel"][idx]
    a["ksr"] = s["ksr"][idx]
    a["rs"] = (s["rs"] if rs is None else rs)[idx]
    return a


def density_epj(idx, s):
    """DensityEPJ::copyFromFP (hdr_density.hpp:66-71)."""
    a = np.zeros(len(idx), abi.DensityEPJ)
    a["id"] = s["id"][idx]
    a["mass"] = s["mass"][idx]
    a["pos"] = s["pos"][idx]
    a["vel"] = s["vel"][idx]
    return a


def _hydro_common(a, idx, s):
    a["id"] = s["id"][idx]
    a["pos"] = s["pos"][idx]
    a["vel"] = s["vel"][idx]
    a["ksr"] = s["ksr"][idx]
    a["hinv"] = 1.0 / s["ksr"][idx]
    a["pres"] = s["pres"][idx]
    a["presc"] = s["pres"][idx] * s["grdh"][idx] / (s["dens"][idx] ** 2)
    a["bswt"] = 0.5 * s["bswt"][idx]
    a["dens"] = s["dens"][idx]
    a["vsnd"] = s["vsnd"][idx]
    a["alph"] = s["alph"][idx]
    a["alphu"] = s["alphu"][idx]
    a["thrm"] = np.maximum(s["uene"][idx] - 0.0, 0.0)   # umin = 0, hdr_hgas.hpp:342
    a["eta"] = s["eta"][idx]
    return a


def hydro_epi(idx, s):
    """HydroEPI::copyFromFP (hdr_hydro.hpp:45-62)."""
    return _hydro_common(np.zeros(len(idx), abi.HydroEPI), idx, s)


def hydro_epj(idx, s):
    """HydroEPJ::copyFromFP (hdr_hydro.hpp:95-113)."""
    a = _hydro_common(np.zeros(len(idx), abi.HydroEPJ), idx, s)
    a["mass"] = s["mass"][idx]
    return a


def gravity_epi(idx, s):
    """GravityEPI::copyFromFP(SPH) (hdr_gravity.hpp:134-137)."""
    a = np.zeros(len(idx), abi.GravityEPI)
    a["pos"] = s["pos"][idx]
    a["eps2"] = (s["ksr"][idx] / units.KSRH) ** 2
    return a


def gravity_epj(idx, s):
    """GravityEPJ::copyFromFP(SPH) (hdr_gravity.hpp:162-166)."""
    a = np.zeros(len(idx), abi.GravityEPJ)
    a["mass"] = s["mass"][idx]
    a["pos"] = s["pos"][idx]
    a["eps2"] = (s["ksr"][idx] / units.KSRH) ** 2
    return a


def concat_walks(items):
    """[(epi, epj), ...] -> (epi_all, epj_all, i_off, j_off) with int64 offsets."""
    i_off = np.zeros(len(items) + 1, np.int64)
    j_off = np.zeros(len(items) + 1, np.int64)
    for k, (a, b) in enumerate(items):
        i_off[k + 1] = i_off[k] + len(a)
        j_off[k + 1] = j_off[k] + len(b)
    epi = np.concatenate([a for a, _ in items]) if items else None
    epj = np.concatenate([b for _, b in items]) if items else None
    return epi, epj, i_off, j_off
