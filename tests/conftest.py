"""Shared test set-up: import paths, the `gpu` marker, workload fixtures."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "thunder-master_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

from fbgpu import synth  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libfbgpu.so")
    config.addinivalue_line("markers", "slow: full-size workloads")


@pytest.fixture(scope="session")
def fdata_root():
    root = os.environ.get("FBGPU_FDATA_ROOT") or os.path.join(ROOT, "_fdata")
    os.makedirs(root, exist_ok=True)
    return root


def workload(name, root, dogs=False, vxc=False):
    """(fdata dir, nZ list, Structure) of a named synthetic workload; dogs:
    the Fdata set with the DOGS charged-shell sub-cells and z-dipole table;
    vxc: the one with the McWEDA exchange-correlation tables."""
    path = synth.fdata_dir_for(name if name in ("si64", "si512", "cho1536", "sic4096") else
                               {"cho_small": "cho1536", "sic_small": "sic4096", "si_vac": "si64",
                                "sic_vac": "sic4096"}[name], root=root, dogs=dogs, vxc=vxc)
    if name in ("si64", "si512", "cho1536", "sic4096"):
        st = synth.structure_for(name)
        nZ = [s.nZ for s in synth.species_for(name)]
    elif name == "cho_small":
        st = synth.random_box([24, 48, 24], 9.0, 1.0, 7, name="CHO96")
        nZ = [s.nZ for s in synth.species_for("cho1536")]
    elif name == "sic_small":
        st = synth.diamond((2, 2, 2), 4.36, 0.1, 11, sp_a=1, sp_b=2, name="SiC64")
        nZ = [14, 6]
    elif name == "si_vac":
        st = synth.diamond((2, 2, 1), 5.43, 0.1, 12, vacancy=0.05, name="Si32v")
        nZ = [14]
    elif name == "sic_vac":
        st = synth.diamond((1, 1, 1), 4.36, 0.1, 13, sp_a=1, sp_b=2, vacancy=0.05, name="SiC8v")
        nZ = [14, 6]
    else:
        raise KeyError(name)
    return path, nZ, st


def random_denmat(nblock, seed):
    """Seeded stand-ins for the density matrices the solver would supply."""
    rng = np.random.default_rng(seed)
    return rng.normal(0.0, 0.1, nblock), rng.normal(0.0, 0.05, nblock)


def symmetric_denmat(orc_sys, norb, seed):
    """A density matrix that is symmetric across neigh_back, as the solver's
    would be (rho_ij(mu,nu) = rho_ji(nu,mu))."""
    rng = np.random.default_rng(seed)
    s = orc_sys
    rho = np.zeros(s.nblock)
    cape = np.zeros(s.nblock)
    N = len(norb)
    for i in range(N):
        for p in range(s.pair_off[i], s.pair_off[i + 1]):
            j = s.neigh_j[p]
            q = s.pair_off[j] + s.neigh_back[p]
            if q < p:
                continue
            a = rng.normal(0.0, 0.1, (norb[i], norb[j]))
            b = rng.normal(0.0, 0.05, (norb[i], norb[j]))
            if p == q:
                a = 0.5 * (a + a.T)
                b = 0.5 * (b + b.T)
            rho[s.blk_off[p]:s.blk_off[p + 1]] = a.T.ravel()
            cape[s.blk_off[p]:s.blk_off[p + 1]] = b.T.ravel()
            rho[s.blk_off[q]:s.blk_off[q + 1]] = a.ravel()
            cape[s.blk_off[q]:s.blk_off[q + 1]] = b.ravel()
    return rho, cape
