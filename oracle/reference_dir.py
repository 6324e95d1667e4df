"""Where the reference tree is mounted (test infrastructure: the reference's kernels are compiled
from it by build_ref.sh, and tests read its case files as text).  Set AFAR_REFERENCE_DIR to use
another location; the default is the mount point of the build container.  Machines without it
(the GPU machines) use the cubins and fixtures already built."""
import os

DEFAULT = "/root/reference"


def reference_dir() -> str:
    return os.environ.get("AFAR_REFERENCE_DIR", DEFAULT)
