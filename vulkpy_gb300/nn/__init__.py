"""
Neural network module (drop-in for vulkpy.nn, vulkpy/nn/__init__.py).

>>> import vulkpy_gb300 as vk
>>> from vulkpy_gb300 import nn
>>> gpu = vk.GPU()
>>> opt = nn.Adam(gpu, lr=1e-4)
>>> net = nn.Sequence([nn.Dense(gpu, 3, 32, w_opt=opt, b_opt=opt), nn.ReLU(),
...                    nn.Dense(gpu, 32, 4, w_opt=opt, b_opt=opt), nn.Softmax()],
...                   nn.CrossEntropyLoss())
"""
from .core import Optimizer, OptimizerState, Loss, Regularizer, Module
from .initializers import Constant, HeNormal
from .optimizers import SGD, SGDState, Adam, AdamState, AdaGrad, AdaGradState
from .layers import Dense, ReLU, Sigmoid, Softmax
from .losses import CrossEntropyLoss, SoftmaxCrossEntropyLoss, MSELoss, HuberLoss, MixLoss
from .regularizers import Lasso, Ridge, Elastic
from .models import Sequence
from .parameters import Parameter
from .data import minibatches
from .grouped import GroupedSequence
