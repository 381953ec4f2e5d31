"""GB300-native RNS-CKKS ciphertext arithmetic (drop-in for the hot path of
Akram275/rns-ckks-rust's `RnsCkksContext`).

The compute path is the CUDA/C++ shared library built from `csrc/` and exposed
through the C ABI declared in `include/rnsckks_gpu.h`; this Python package is a
thin host-side mirror of the reference API over that ABI.
"""
from . import params  # noqa: F401
from .params import RnsCkksParams, RnsPrime  # noqa: F401
from ._lib import RcError, build, lib  # noqa: F401


def __getattr__(name):
    # the GPU-facing API (torch-backed) is imported on first use
    if name in ("context", "RnsCkksContext", "RnsCiphertext", "RnsQuadraticCiphertext", "RnsPolynomial",
                "RnsKeySwitchingKey", "RnsRotationKey", "Sampler", "galois_element_for_rotation",
                "to_device", "to_host"):
        import importlib
        _c = importlib.import_module(__name__ + ".context")
        return _c if name == "context" else getattr(_c, name)
    raise AttributeError(name)
