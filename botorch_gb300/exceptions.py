"""Exception types with the reference's names and meaning.

``NotPSDError`` / ``NanError`` mirror linear_operator.utils.errors (raised by
psd_safe_cholesky and by botorch/utils/low_rank.py:162-171);
``UnsupportedError`` mirrors botorch/exceptions/errors.py.
"""


class BotorchError(Exception):
    """Base exception (botorch/exceptions/errors.py:16)."""


class UnsupportedError(BotorchError):
    """Requested configuration is not supported by this path."""


class NotPSDError(RuntimeError):
    """psd_safe_cholesky failed after all jitter retries."""


class NanError(RuntimeError):
    """NaN input to a Cholesky or non-finite posterior samples."""


class BotorchWarning(Warning):
    """Base warning (botorch/exceptions/warnings.py:12); issued, as in the reference, when
    the cached-root sampling of qLogNEI falls back to joint sampling."""
