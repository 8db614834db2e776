"""Form factor models (sparrowpy/form_factor): `universal` and `kang`, on the GPU.

The package keeps the reference's public names: patch2patch_ff_universal
(universal.py) and patch2patch_ff_kang (kang.py), and in the submodules the
pair form factor and the point-source / point-receiver factors that the
reference's tests call.
"""
from . import kang, universal
from .kang import patch2patch_ff_kang
from .universal import patch2patch_ff_universal

__all__ = ["patch2patch_ff_universal", "patch2patch_ff_kang"]
