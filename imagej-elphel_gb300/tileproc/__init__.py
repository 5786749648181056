"""GB300 tile processor: host-side mirror of the imagej-elphel GPUTileProcessor /
ImageDtt call surface over the C ABI in include/tp.h (libtp.so)."""
from . import _lib
from .processor import GPUTileProcessor

__all__ = ["GPUTileProcessor", "_lib"]
