"""Element descriptors (the reference's diffmpm/element.py).

``Quadrilateral4Node`` describes the structured 2-D mesh the GPU kernels work
on: node ``id = j (nx + 1) + i`` at ``(i hx, j hy)`` (float32, rounded once as
the reference forms them, element.py:663-690), element ``e`` with nodes
``[ll, ll + 1, ll + nx + 2, ll + nx + 1]``, ``ll = (e // nx)(nx + 1) + e % nx``
(element.py:692-723).  Shape functions, gradients, scatters and gathers are
evaluated by the CUDA kernels.
"""
from __future__ import annotations

import numpy as np

from .node import Nodes


class _Element:
    ndim = 2

    def id_to_node_ids(self, id):
        raise NotImplementedError


class Quadrilateral4Node(_Element):
    """2-D 4-node quadrilateral elements (diffmpm/element.py:603-909)."""

    ndim = 2

    def __init__(self, nelements, total_elements, el_len, constraints, nodes=None,
                 concentrated_nodal_forces=(), initialized=None, volume=None):
        nel = np.asarray(nelements, dtype=np.int64).reshape(-1)
        if nel.size != 2 or (nel < 1).any():
            raise ValueError(f"nelements must be two positive integers, found {nelements}")
        self.nelements = (int(nel[0]), int(nel[1]))
        self.total_elements = int(total_elements)
        if self.total_elements != self.nelements[0] * self.nelements[1]:
            raise ValueError("total_elements must equal nx * ny")
        self.el_len = np.broadcast_to(np.asarray(el_len, dtype=np.float32).reshape(-1), (2,)).copy()
        nx, ny = self.nelements
        if nodes is None:
            xs = np.arange(nx + 1).astype(np.float32) * self.el_len[0]
            ys = np.arange(ny + 1).astype(np.float32) * self.el_len[1]
            loc = np.stack(np.broadcast_arrays(xs[None, :], ys[:, None]), axis=-1).reshape(-1, 1, 2)
            self.nodes = Nodes((nx + 1) * (ny + 1), loc)
        else:
            self.nodes = nodes
        self.constraints = list(constraints)
        self.concentrated_nodal_forces = list(concentrated_nodal_forces)
        self.volume = (np.ones((self.total_elements, 1, 1), dtype=np.float32)
                       if volume is None else np.asarray(volume, dtype=np.float32))

    def id_to_node_ids(self, id):
        nx = self.nelements[0]
        e = np.asarray(id, dtype=np.int64)
        ll = (e // nx) * (nx + 1) + e % nx
        return np.asarray([ll, ll + 1, ll + nx + 2, ll + nx + 1]).reshape(4, 1)


class Linear1D(_Element):
    """1-D two-node line elements (diffmpm/element.py:343-600), nodes at
    float(i) * el_len.  The GPU step (csrc/mpm_line.cu) takes the element
    volume as its length and the strain rate as [dN/dx . v, 0, 0, 0, 0, 0],
    where the reference's own 1-D code does not run as written
    (element.py:543-546, particle.py:304-305)."""

    ndim = 1

    def __init__(self, nelements, total_elements, el_len, constraints, nodes=None,
                 concentrated_nodal_forces=(), initialized=None, volume=None):
        self.nelements = int(np.asarray(nelements).reshape(-1)[0])
        self.total_elements = self.nelements
        self.el_len = np.float32(np.asarray(el_len).reshape(-1)[0])
        self.nodes = nodes if nodes is not None else Nodes(
            self.nelements + 1, (np.arange(self.nelements + 1).astype(np.float32) * self.el_len).reshape(-1, 1, 1))
        self.constraints = list(constraints)
        self.concentrated_nodal_forces = list(concentrated_nodal_forces)
        self.volume = (np.ones((self.total_elements, 1, 1), dtype=np.float32)
                       if volume is None else np.asarray(volume, dtype=np.float32))
