"""Shape-annotated type aliases with the reference's names (torchfsm/_type.py).

``SpatialTensor["B C H ..."]`` is ``typing.Annotated[torch.Tensor, "B C H ..."]`` (likewise
``FourierTensor`` for spectra and ``SpatialArray`` / ``FourierArray`` over ``numpy.ndarray``):
annotations only, never instantiated. ``ValueList[T]`` is ``Union[T, List[T]]``.
"""

from __future__ import annotations

from typing import Annotated, List, Union

import numpy as np
from torch import Tensor


class _ShapeAlias:
    """Base of the shape-annotated aliases: subscripting gives Annotated[base, shape]."""

    __slots__ = ()
    _base: type = object

    def __new__(cls, *args, **kwargs):
        raise TypeError(f"{cls.__name__} is a type annotation and cannot be instantiated")

    def __class_getitem__(cls, shape: str):
        return Annotated[cls._base, shape]


class SpatialTensor(_ShapeAlias):
    _base = Tensor


class FourierTensor(_ShapeAlias):
    _base = Tensor


class SpatialArray(_ShapeAlias):
    _base = np.ndarray


class FourierArray(_ShapeAlias):
    _base = np.ndarray


class ValueList:
    """``ValueList[T]``: a value of type T or a list of them."""

    __slots__ = ()

    def __new__(cls, *args, **kwargs):
        raise TypeError("ValueList is a type annotation and cannot be instantiated")

    def __class_getitem__(cls, item):
        return Union[item, List[item]]
