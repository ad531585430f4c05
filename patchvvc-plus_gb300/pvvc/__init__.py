"""pvvc -- GB300-native patchVVC per-patch codec path (Python mirror of the C ABI
in include/pvvc_gb300.h; the work runs in libpvvc_gb300.so)."""
from ._lib import LIB_PATH, STATUS, PvvcError, build_library, check, lib  # noqa: F401
from .codec import Decoder, Graph, Plan, autotune, encode_patch_gop, rlgr_decode, rlgr_encode  # noqa: F401
from .frame import Batch, Frame, concat_batches, pack_frames, parse_frame, parse_slice, write_frame  # noqa: F401
from .synth import Synth, config  # noqa: F401
from .serve import Server, playback  # noqa: F401
