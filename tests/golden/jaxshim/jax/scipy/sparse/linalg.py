"""Matrix-free CG/BiCGSTAB stand-ins built on SciPy's LinearOperator."""

import numpy as _np


def _solve(method, A, b, x0=None, tol=1e-5, atol=0.0, maxiter=None, M=None):
    import scipy.sparse.linalg as sla
    b = _np.asarray(b)
    shape = b.shape
    n = b.size
    op = sla.LinearOperator((n, n), matvec=lambda v: _np.asarray(A(v.reshape(shape))).ravel())
    pre = None if M is None else sla.LinearOperator(
        (n, n), matvec=lambda v: _np.asarray(M(v.reshape(shape))).ravel())
    x, info = method(op, b.ravel(), x0=None if x0 is None else _np.asarray(x0).ravel(),
                     rtol=tol, atol=atol, maxiter=maxiter, M=pre)
    from ... import numpy as jnp
    return jnp.asarray(x.reshape(shape)), info


def cg(A, b, x0=None, *, tol=1e-5, atol=0.0, maxiter=None, M=None):
    import scipy.sparse.linalg as sla
    return _solve(sla.cg, A, b, x0, tol, atol, maxiter, M)


def bicgstab(A, b, x0=None, *, tol=1e-5, atol=0.0, maxiter=None, M=None):
    import scipy.sparse.linalg as sla
    return _solve(sla.bicgstab, A, b, x0, tol, atol, maxiter, M)
