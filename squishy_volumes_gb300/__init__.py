"""GB300 implementation of the Squishy Volumes MPM substep.

The compute path is libsquishy_volumes_cuda.so (hand-written CUDA for
sm_103a behind the C ABI in include/squishy_volumes_cuda.h); this package is
its host-side mirror of the reference's backend interface.
"""

from .state import (  # noqa: F401
    Canceled,
    CudaState,
    EnergyError,
    Extras,
    FrameData,
    FrameInput,
    GridNodes,
    Harness,
    InputConsts,
    IoState,
    Particles,
    RunParameters,
    ZeroTimeStep,
    sort_pairs,
)
