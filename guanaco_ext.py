"""guanaco_ext: the name of the reference's compiled extension module
(src/guanaco/detail/ext/guanaco_ext.cpp:32-37), here over this library's C ABI.

The reference's Python package takes its whole native interface from it with
``from guanaco_ext import *`` (src/guanaco/detail/__init__.py:21).  With this
file's directory on the import path ahead of the reference's build, that
package's device path (device="gpu") -- recon per Y row, corr per tilt, the
CTF class and the unit conversions -- runs on the GB300 library unchanged.
Names, arguments, defaults and assertion messages are those of the
reference's bindings (guanaco_gb300.detail); the CPU path (device="cpu")
raises, as everywhere in this library.
"""
from guanaco_gb300.detail import *  # noqa: F401,F403
from guanaco_gb300.detail import __all__  # noqa: F401
