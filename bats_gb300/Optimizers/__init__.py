from .GradientDescentOptimizer import GradientDescentOptimizer
from .AdamOptimizer import AdamOptimizer
from .NAdamOptimizer import NAdamOptimizer
