"""Shared helpers of the test suite (parity metrics, mesh variants)."""
import numpy as np
import scipy.sparse as sp

from elastic_gb300 import meshgen as M


def full_matrix(ia, ja, ad, al):
    """K = D + L + L^T as a scipy CSR matrix from CSRC arrays (1-based ia/ja)."""
    n = ia.shape[0] - 1
    rows = np.repeat(np.arange(n), np.diff(ia))
    L = sp.csr_matrix((al, (rows, np.asarray(ja) - 1)), shape=(n, n))
    return (L + L.T + sp.diags(ad)).tocsr()


def relabel_nodes(m, seed):
    """The same mesh with its nodes numbered in a random order."""
    rng = np.random.default_rng(seed)
    newnum = rng.permutation(m.nnode)
    inv = np.argsort(newnum)
    m2 = M.Mesh(ndm=m.ndm, ndf=m.ndf, nen=m.nen, x=m.x[inv].copy(), ix=m.ix.copy(), ie=m.ie,
                e=m.e, id=m.id[inv].copy(), f=m.f[inv].copy(), name=m.name + "_relabelled")
    m2.ix[:, :m.nen] = newnum[m.ix[:, :m.nen] - 1] + 1
    return m2


def two_components(m):
    """Two disjoint copies of a mesh in one model (two graph components)."""
    n = m.nnode
    ix2 = m.ix.copy()
    ix2[:, :m.nen] += n
    x2 = m.x.copy()
    x2[:, 0] += 10.0
    return M.Mesh(ndm=m.ndm, ndf=m.ndf, nen=m.nen, x=np.vstack([m.x, x2]),
                  ix=np.vstack([m.ix, ix2]), ie=m.ie, e=m.e, id=np.vstack([m.id, m.id]),
                  f=np.vstack([m.f, m.f]), name=m.name + "_x2")


def rollers(m, axis=0):
    """The same mesh with the normal dof of the nodes on the face x_axis = min
    fixed (rollers): those nodes are only partly fixed, so the equations no
    longer come in whole node blocks."""
    m2 = M.Mesh(ndm=m.ndm, ndf=m.ndf, nen=m.nen, x=m.x, ix=m.ix, ie=m.ie, e=m.e,
                id=m.id.copy(), f=m.f.copy(), name=m.name + "_rollers")
    face = np.isclose(m.x[:, axis], m.x[:, axis].min())
    m2.id[face, axis] = 1
    m2.f[face, axis] = 0.0
    return m2


def row_scaled_error(ia, a_ref, a_got, ad_ref, ad_got):
    """max |delta| over the entries of each row, divided by the row's largest
    |entry| (diagonal included): the assembly parity metric."""
    n = ia.shape[0] - 1
    lens = np.diff(ia)
    rows = np.repeat(np.arange(n), lens)
    rowmax = np.abs(ad_ref).copy()
    if a_ref.size:
        # rows are contiguous runs of al: the max of each non-empty run
        full = lens > 0
        runmax = np.maximum.reduceat(np.abs(a_ref), np.asarray(ia[:-1])[full] - 1)
        rowmax[full] = np.maximum(rowmax[full], runmax)
    err = np.abs(ad_ref - ad_got) / rowmax
    if a_ref.size:
        err_l = np.abs(a_ref - a_got) / rowmax[rows]
        return float(max(err.max(), err_l.max()))
    return float(err.max())


def rel_inf(ref, got):
    """||got - ref||_inf / ||ref||_inf."""
    ref = np.asarray(ref)
    d = np.abs(np.asarray(got) - ref).max()
    s = np.abs(ref).max()
    return float(d / s) if s > 0 else float(d)
