"""Host side of failure detection (no GPU): the device error word's bits map
to the documented exceptions, and the product raises instead of falling back
when the library is missing."""
import pytest


@pytest.mark.parametrize("word,exc", [(1, "DeviceTimeout"), (2, "NonFiniteError"), (3, "DeviceTimeout"),
                                      (8, "FlowketError")])
def test_check_device_maps_status_bits(monkeypatch, word, exc):
    from flowket_gb300 import _lib
    monkeypatch.setattr(_lib, "device_status", lambda clear=True: word)
    with pytest.raises(getattr(_lib, exc)):
        _lib.check_device("test")


def test_check_device_passes_on_zero(monkeypatch):
    from flowket_gb300 import _lib
    monkeypatch.setattr(_lib, "device_status", lambda clear=True: 0)
    _lib.check_device("test")


def test_missing_library_raises(monkeypatch, tmp_path):
    from flowket_gb300 import _lib
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "absent.so"))
    with pytest.raises(_lib.FlowketError, match="no CPU fallback"):
        _lib.load()
