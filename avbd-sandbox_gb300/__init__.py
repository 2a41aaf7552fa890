"""GB300-native AVBD world step: CUDA backend behind a C ABI, plus the host-side
mirror of the reference's `GpuBackend` interface."""
from . import abi, scene  # noqa: F401
