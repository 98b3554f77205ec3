"""adpy.config stand-in: the reference calls set_config(module) at import (adFVM/config.py:119-120)."""


def set_config(module):
    return None


def get_sources():
    return []


def get_include_dirs():
    return []
