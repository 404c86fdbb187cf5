"""mbx: host-side mirror of the reference's MB-pol force path on top of libmbx.so."""
from . import systems  # noqa: F401
