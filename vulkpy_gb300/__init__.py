"""
vulkpy_gb300: vulkpy's array engine on NVIDIA GB300 (sm_103a).

Drop-in for ``import vulkpy as vk``:

>>> import vulkpy_gb300 as vk
>>> gpu = vk.GPU()
>>> a = vk.Array(gpu, data=[1, 2, 3])
>>> b = vk.Array(gpu, data=[3, 3, 3])
>>> c = a + b
>>> print(c)
[4. 5. 6.]

The native library (CUDA kernels behind a C ABI, include/vulkpy_gb300.h) is
required; importing without it raises ImportError.
"""
from .vkarray import GPU, U32Array, Shape, Array, zeros
from . import random
from . import nn
from . import graph
from . import fusion
from . import autotune as _autotune

_autotune.load_table()

__all__ = ["GPU", "U32Array", "Shape", "Array", "zeros", "random", "nn"]
