"""Tests reach the C ABI through the package's ctypes binding."""
from cppe_gb300.capi import *  # noqa: F401,F403
from cppe_gb300.capi import declared_functions, lib, last_error, LIB_PATH  # noqa: F401
