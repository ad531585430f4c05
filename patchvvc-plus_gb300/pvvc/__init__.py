"""pvvc -- GB300-native patchVVC per-patch codec path (Python mirror of the C ABI
in include/pvvc_gb300.h; the work runs in libpvvc_gb300.so)."""
from ._lib import LIB_PATH, STATUS, PvvcError, build_library, check, lib  # noqa: F401
from .codec import (Decoder, Encoder, Graph, Plan, autotune, encode_patch_gop, patch_leaf_yuv, rlgr_decode,  # noqa: F401
                    rlgr_encode)
from .frame import Batch, Frame, concat_batches, pack_frames, parse_frame, parse_slice, write_frame  # noqa: F401
from .synth import Synth, config  # noqa: F401
from .serve import Server, playback  # noqa: F401
from . import zstd  # noqa: F401
