"""Utilities (names of vulkpy/util.py).

``enable_debug`` replaces the Vulkan validation-layer switch
(vulkpy/util.py:17-54) with CUDA-side checking: every op is followed by a
stream synchronisation and a read of the device error word, so a failing
launch or an out-of-range gather index raises at the op that caused it.
"""
from __future__ import annotations

import logging
import os

logger = logging.getLogger("vulkpy_gb300")

_DEBUG = {"sync": os.environ.get("VULKPY_GB300_DEBUG", "0") not in ("", "0")}


def enable_debug(*, validation: bool = True, api_dump: bool = True):
    """Turn on synchronous error checking after every op.

    Parameters
    ----------
    validation : bool, optional
        If ``True`` (default), synchronise and check the device error word
        after every op.
    api_dump : bool, optional
        If ``True`` (default), log every native call at DEBUG level.
    """
    logging.basicConfig(level=logging.DEBUG)
    logger.setLevel(logging.DEBUG)
    logger.debug("Enable debug mode")
    _DEBUG["sync"] = bool(validation)
    _DEBUG["dump"] = bool(api_dump)


def disable_debug():
    """Turn synchronous checking off again."""
    _DEBUG["sync"] = False
    _DEBUG["dump"] = False


def debug_enabled() -> bool:
    return bool(_DEBUG.get("sync"))


def getShader(name: str) -> str:
    """Kept for API compatibility: there are no shader files; returns ``name``."""
    return name
