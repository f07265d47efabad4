"""cuda_device: the reference's device module (sqaodpy/sqaod/cuda/src/cuda_device.cpp),
used by sqaodpy/sqaod/cuda/device.py: new(), initialize(obj, devno),
finalize(obj), delete(obj).  A device object carries its device number; a
solver assigned to it runs its work on that device."""
import ctypes

from .._lib import call, lib


class _Device:
    def __init__(self):
        self.devno = None


def new():
    return _Device()


def initialize(obj, devno):
    if not isinstance(obj, _Device):
        raise RuntimeError("invalid device object.")
    devno = int(devno)
    call(lib().sq103_device_set, ctypes.c_int(devno))
    obj.devno = devno


def finalize(obj):
    if not isinstance(obj, _Device):
        raise RuntimeError("invalid device object.")
    obj.devno = None


def delete(obj):
    if not isinstance(obj, _Device):
        raise RuntimeError("invalid device object.")


def assign(devobj):
    """Makes the device of `devobj` current (the solvers' assign_device)."""
    if not isinstance(devobj, _Device) or devobj.devno is None:
        raise RuntimeError("the device is not initialized.")
    call(lib().sq103_device_set, ctypes.c_int(devobj.devno))
