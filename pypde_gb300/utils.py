"""Argument helpers with the reference's behaviour (pypde/utils.py)."""
import inspect
import sys

from numpy import array

BOUNDARIES = {"transitive": 0, "periodic": 1}


def nargs(func):
    return len(inspect.signature(func).parameters)


def parse_boundary_types(boundaryTypes, ndim):
    """'transitive'/'periodic' or a list of them -> int32 codes
    (pypde/utils.py:37-66).  Invalid input prints the reference's message and
    exits with status 1, as the reference does."""
    errMsg = ('boundaryTypes must be a string from {"transitive", "periodic"} '
              'or a list of such strings, of length equal to the number of '
              'dimensions of the domain.')
    if isinstance(boundaryTypes, str):
        if boundaryTypes not in BOUNDARIES:
            print(errMsg)
            sys.exit(1)
        ret = [BOUNDARIES[boundaryTypes]] * ndim
    elif isinstance(boundaryTypes, list):
        if len(boundaryTypes) != ndim or any(b not in BOUNDARIES for b in boundaryTypes):
            print(errMsg)
            sys.exit(1)
        ret = [BOUNDARIES[b] for b in boundaryTypes]
    else:
        print(errMsg)
        sys.exit(1)
    return array(ret, dtype="int32")
