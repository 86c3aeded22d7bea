"""Exceptions and warnings of the Pysic API.

Same class names, meanings and warning levels as pysic/utility/error.py:32-315
of the reference, so user code that catches them keeps working.
"""
import sys


class Warning:  # noqa: A001 - name kept from pysic/utility/error.py:6
    """Global warning level: messages with a level below it are printed
    (pysic/utility/error.py:6-48)."""

    level = 10


class WarningInterruptException(Exception):
    """Raised when a warning of level 0 is issued (pysic/utility/error.py:50-64)."""


def set_warning_level(level):
    """Set the level at and above which warnings are suppressed."""
    Warning.level = level


def warn(message, level):
    """Print a warning if its level is below the global level
    (pysic/utility/error.py:135-150)."""
    if level == 0:
        raise WarningInterruptException(message)
    if level < Warning.level:
        sys.stderr.write("*** pysic warning (level {0}) ***\n{1}\n".format(level, message))


def error(message):
    sys.stderr.write("*** pysic error ***\n{0}\n".format(message))


class InvalidPotentialError(Exception):
    """Invalid potential definition (pysic/utility/error.py:164-183)."""


class InvalidCoordinatorError(Exception):
    """Invalid coordinator (pysic/utility/error.py:185-204)."""


class InvalidParametersError(Exception):
    """Invalid parameters (pysic/utility/error.py:206-225)."""


class InvalidSummationError(Exception):
    """Invalid Coulomb summation (pysic/utility/error.py:227-246)."""


class InvalidRelaxationError(Exception):
    """Invalid charge relaxation (pysic/utility/error.py:248-267)."""


class MissingAtomsError(Exception):
    """Atoms missing from the calculator (pysic/utility/error.py:269-282)."""


class MissingNeighborsError(Exception):
    """Neighbour lists missing (pysic/utility/error.py:284-300)."""


class LockedCoreError(Exception):
    """Engine state cannot be changed as requested (pysic/utility/error.py:302-315)."""


class EngineError(RuntimeError):
    """A call into the GB300 engine returned an error status.

    ``status`` is the integer code of the C ABI (include/pysic_gb300.h)."""

    def __init__(self, status, message):
        RuntimeError.__init__(self, "GB300 engine error {0}: {1}".format(status, message))
        self.status = status
