"""GB300-native NuSiF hot path: host-side mirror of the reference interface.

The compute path is the CUDA library ``lib/libnusif_gb300.so`` (C ABI in
include/nusif_gb300.h); this package loads it with ctypes and drives the
reference time loop. Importing the package does not need a GPU; calls that
launch kernels do.
"""
from .abi import NusifError, load_library, check, LIB_PATH  # noqa: F401
from .params import write_par, cavity, config1, config2, channel, DCAVITY, CANAL  # noqa: F401
from .sim import Simulation, StepInfo  # noqa: F401
from .batch import Batch, InstanceStats  # noqa: F401
from .unet import UNet  # noqa: F401
