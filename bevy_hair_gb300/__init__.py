"""bevy_hair_gb300: bevy_hair's per-frame strand-hair pipeline on GB300 (sm_103a).

The compute passes of ``hair_pass`` (src/render/pass.rs:259-657) run as
hand-written CUDA kernels behind the C ABI in ``include/hairgb.h``; this
package holds the Python side of the host: ctypes bindings (``abi``), the
uniform math of pass.rs (``host``), grooms and the baker (``groom``), the
pass orchestration (``pipeline``) and the benchmark scenes (``configs``).
"""
from . import abi, host, groom  # noqa: F401

__all__ = ["abi", "host", "groom"]
