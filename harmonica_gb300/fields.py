"""
Field names and codes shared by the Python API and the C ABI.

The names are harmonica's ``FIELDS`` (``src/harmonica/_forward/prisms/gravity.py:37-48``);
the codes are the bit positions of the ``field_mask`` argument of the C ABI
(``include/harmonica_gb300.h``).
"""

FIELDS = ("potential", "g_e", "g_n", "g_z", "g_ee", "g_nn", "g_zz", "g_en", "g_ez", "g_nz")
FIELD_CODES = {name: code for code, name in enumerate(FIELDS)}
TENSOR_FIELDS = frozenset(("g_ee", "g_nn", "g_zz", "g_en", "g_ez", "g_nz"))


def field_mask(fields):
    """Bit mask of the C ABI for an iterable of field names."""
    mask = 0
    for f in fields:
        mask |= 1 << FIELD_CODES[f]
    return mask
