"""Aperture windows: the reference's C keep-condition, parsed to a stack program.

The reference pastes the window text into ``if ({window} == 0) x = NAN;``
(ufo/elements.py:517-518) without parentheses around ``window``, so the C
operator precedence of the concatenated text decides what is tested (for
``'a && b'`` the test is ``a && (b == 0)``).  This module parses exactly that
concatenated text with C precedence and C's int/double typing and emits a
postfix program that the kernels evaluate per particle; the grammar and the
typing are those of :mod:`ufo_gb300.cexpr` (without ``parameters[]``).
Anything else raises ``NotImplementedError``: the reference accepted arbitrary
OpenCL C there, which a data-driven kernel cannot run.
"""
from . import cexpr as _x
from .cexpr import (PUSH, VAR, NEG, NOT, ADD, SUB, MUL, DIV, IDIV, IMOD, LT, LE, GT,  # noqa: F401
                    GE, EQ, NE, AND, OR, FABS, SQRT, SEL, VARS, INT_VARS)

MAX_STACK = 16


def compile_window(window):
    """Postfix program for the reference's loss test ``{window} == 0``.
    Returns a list of (opcode, value); the particle is lost when it
    evaluates to non-zero."""
    code, _, _ = _x.compile_expr(f'{window} == 0', 'aperture window')
    if _x.depth(code) > MAX_STACK:
        raise NotImplementedError('aperture window: expression too deep')
    return code


def evaluate(code, x=0., px=0., y=0., py=0., z=0., dp=0., oodppo=1., turn=0):
    """Reference evaluator of a compiled window (used by tests): True when
    the particle is lost."""
    return _x.evaluate(code, (x, px, y, py, z, dp, oodppo, turn)) != 0
