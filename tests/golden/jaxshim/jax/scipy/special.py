from scipy.special import gammaln as _gammaln

from ..numpy import _wrap


def gammaln(x):
    return _wrap(_gammaln(x))
