"""fastxc_gb300: GB300-native (sm_103a) ambient-noise correlation hot path.

The compute lives in ``lib/libfastxc_gb300.so`` (C ABI: ``include/fastxc_gb300.h``);
this package is the host-side mirror of the reference's stage interface.
"""

from ._lib import FxcError, FxcLibraryMissing, lib  # noqa: F401

__version__ = "0.1.0"
