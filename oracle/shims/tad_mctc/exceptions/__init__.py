"""Exception types raised by dxtb's input checks (``types/base.py:518-842``)."""


class DeviceError(RuntimeError):
    pass


class DtypeError(ValueError):
    pass


__all__ = ["DeviceError", "DtypeError"]
