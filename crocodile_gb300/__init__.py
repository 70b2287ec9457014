"""GB300-native convolutional gridding for crocodile (SKA-ScienceDataProcessor).

``crocodile_gb300.synthesis`` is a drop-in replacement of ``crocodile.synthesis``
whose gridding path runs in hand-written sm_103a kernels
(``libcrocodile_gb300.so``, C ABI in ``include/crocodile_gb300.h``).
"""

__version__ = "0.1.0"
