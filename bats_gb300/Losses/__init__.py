from .TTFSSoftmaxCrossEntropy import TTFSSoftmaxCrossEntropy
from .SpikeCountClassLoss import SpikeCountClassLoss
from .SpikeCountLoss import SpikeCountLoss
from .SpikeTimeLoss import SpikeTimeLoss
