"""Shared pytest configuration.  GPU tests are marked ``gpu``; the rest run on CPU."""

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")


_ORACLES: dict = {}


def _oracle(arith: str):
    from oracle import Oracle

    if arith not in _ORACLES:
        _ORACLES[arith] = Oracle(arith)
    return _ORACLES[arith]


def _set_library_arith(arith: str):
    import isoext_gb300 as iso

    iso.set_arithmetic(arith)


@pytest.fixture(params=["nvcc", "host"])
def oracle(request):
    """The oracle in one reading of isoext's arithmetic, with the library set to
    the same reading: every test that compares against it runs for isoext's CUDA
    build (nvcc, the library's default) and for its host build."""
    _set_library_arith(request.param)
    yield _oracle(request.param)
    _set_library_arith("nvcc")


@pytest.fixture
def host_oracle():
    """The oracle in the host build's reading, which the reference's host build
    (oracle/_ref) and the golden fixtures made from it compute."""
    return _oracle("host")


@pytest.fixture
def host_arith():
    """The library in the host build's reading, for comparisons with fixtures
    made by the reference's host build."""
    _set_library_arith("host")
    yield
    _set_library_arith("nvcc")


@pytest.fixture(scope="session")
def reference():
    from oracle import Reference

    try:
        return Reference()
    except FileNotFoundError:
        pytest.skip("the reference's host build is not available here")
