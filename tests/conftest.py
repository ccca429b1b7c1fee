"""Shared test setup.

Markers: ``gpu`` tests need a CUDA GPU (sm_103a) and call the product through
its C-ABI; everything else runs on CPU.  The oracle (oracle/) is the checker;
the product is navier-stokes-solvers_gb300/libns_gb300.so.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "navier-stokes-solvers_gb300"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the sm_103a library")


def golden(name: str):
    return np.load(os.path.join(GOLDEN, name))


def rel_l2(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))


def grid(n, L=2 * np.pi):
    return np.arange(n) * L / n


def tg_vorticity(nx, ny):
    return 2.0 * np.sin(grid(nx))[None, :] * np.sin(grid(ny))[:, None]


def random_field(nx, ny, seed, kcut_frac=1.0 / 6):
    """Seeded smooth random field: |k| <= min(nx,ny)*kcut_frac (same recipe as the fixtures)."""
    rng = np.random.default_rng(seed)
    f = rng.standard_normal((ny, nx))
    fh = np.fft.rfft2(f)
    kx = np.fft.rfftfreq(nx, 1.0 / nx)[None, :]
    ky = np.fft.fftfreq(ny, 1.0 / ny)[:, None]
    fh[np.sqrt(kx ** 2 + ky ** 2) > min(nx, ny) * kcut_frac] = 0
    return np.fft.irfft2(fh, s=(ny, nx))


@pytest.fixture(scope="session")
def port():
    import oracle

    oracle.build(ref=False)
    return oracle.load("port")


@pytest.fixture(scope="session")
def nsgb():
    import nsgb as m

    m.load()
    return m
