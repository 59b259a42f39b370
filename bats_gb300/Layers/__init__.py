from .InputLayer import InputLayer
from .LIFLayer import LIFLayer
from .ConvInputLayer import ConvInputLayer
from .ConvLIFLayer import ConvLIFLayer, LIFLayerConv
from .PoolingLayer import PoolingLayer
