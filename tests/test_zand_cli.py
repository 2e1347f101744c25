"""Host-side pieces of the ``zand`` driver that need no GPU."""
import pytest

from zandpack_gb300.zand import _install_standins, parse_dir


def test_parse_dir_like_reference():
    assert parse_dir(["Dir=/tmp/x"]) == "/tmp/x"
    assert parse_dir(["Dir = /tmp/y"]) == "/tmp/y"
    assert parse_dir([]) is None
    with pytest.raises(AssertionError):
        parse_dir(["Dir=/a", "Dir=/b"])
    with pytest.raises(AssertionError):
        parse_dir(["Dir"])


def test_standins_for_reference_imports():
    _install_standins()
    from Zandpack.td_constants import hbar
    from Zandpack.Loader import load_dictionary  # noqa: F401
    from mpi4py import MPI
    assert abs(hbar - 0.6582119569) < 1e-12
    assert MPI.COMM_WORLD.Get_rank() == 0
