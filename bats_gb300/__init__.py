"""bats_gb300: the BATS event-based LIF simulation and exact multi-spike backpropagation on GB300
(sm_103a) kernels behind a C ABI, with the reference's Python API (Network, layers, losses, Adam)."""
from .AbstractLayer import AbstractLayer
from .AbstractOptimizer import AbstractOptimizer
from .AbstractLoss import AbstractLoss
from .AbstractConvLayer import AbstractConvLayer
from .Network import Network
from .Losses import *  # noqa: F401,F403
from ._lib import BatsError, load as load_library

__all__ = ["AbstractLayer", "AbstractOptimizer", "AbstractLoss", "AbstractConvLayer", "Network", "BatsError",
           "load_library", "TTFSSoftmaxCrossEntropy", "SpikeCountClassLoss", "SpikeCountLoss", "SpikeTimeLoss"]
