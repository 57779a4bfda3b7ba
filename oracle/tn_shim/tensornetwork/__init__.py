"""Restatement of the subset of TensorNetwork 0.2.1 that mpsim calls.

Test infrastructure only.  ``tensornetwork==0.2.1`` (pinned by the
reference's requirements.txt:2) is not installed in this environment and there
is no network, so this module restates the library's published behaviour for
exactly the calls mpsim makes (mpsim/core.py, mpsim/gates.py):

  Node, Edge, connect, contract, contract_between, flatten_edges_between,
  split_node, split_node_full_svd, copy, check_connected, get_shared_edges.

It lets ``tests/golden/make_golden.py`` execute the reference's own, unmodified
``core.py`` on seeded circuits and its own unit tests, which pins the NumPy
oracle (oracle/ref_mps.py) to the reference's control flow.

Semantics restated from the library's documentation and numpy backend:
* A new Node gets one dangling Edge per axis; the default node name is
  "__unnamed_node__".
* ``connect`` replaces two dangling edges with one edge (node1 = first edge's
  node, node2 = second edge's node).
* ``contract_between`` tensordots over every shared edge; the result keeps
  node1's free edges in axis order followed by node2's.
* ``flatten_edges_between`` merges all shared edges into one edge placed last
  on both nodes, flattening in one common edge order.
* ``svd_decomposition`` reshapes to (prod(left), prod(right)), calls
  ``np.linalg.svd(full_matrices=False)``, keeps
  ``min(max_singular_values, count(trunc_errs > max_truncation_err))`` values
  where trunc_errs = sqrt(cumsum(s[::-1]**2)), casts s to the tensor's dtype and
  returns the discarded values.
* ``split_node`` gives U*sqrt(S), sqrt(S)*V^H; ``split_node_full_svd`` gives
  U, diag(S), V^H as three connected nodes.
* Nodes consumed by a contraction or split keep their tensors and get fresh
  dangling edges (mpsim relies on this to apply one gate node to many sites,
  core.py:941-948).
"""

import numpy as np

__version__ = "0.2.1-restated-subset"


class Edge:
    def __init__(self, node1, axis1, name=None, node2=None, axis2=None):
        self.node1 = node1
        self.axis1 = axis1
        self.node2 = node2
        self.axis2 = axis2
        self.name = name if name is not None else "__unnamed_edge__"

    def is_dangling(self):
        return self.node2 is None

    @property
    def dimension(self):
        return self.node1.tensor.shape[self.axis1]

    def get_nodes(self):
        return [self.node1, self.node2]

    def update_axis(self, old_axis, old_node, new_axis, new_node):
        if self.node1 is old_node and self.axis1 == old_axis:
            self.node1, self.axis1 = new_node, new_axis
        elif self.node2 is old_node and self.axis2 == old_axis:
            self.node2, self.axis2 = new_node, new_axis
        else:
            raise ValueError("Edge does not reference the given node/axis.")

    def __repr__(self):
        return f"Edge({self.name})"


class Node:
    def __init__(self, tensor, name=None, axis_names=None, backend=None):
        if isinstance(tensor, Node):
            tensor = tensor.tensor
        self._tensor = np.asarray(tensor)
        self.name = name if name is not None else "__unnamed_node__"
        if axis_names is None:
            axis_names = [None] * self._tensor.ndim
        self.axis_names = list(axis_names)
        self.edges = [Edge(self, i, name=axis_names[i])
                      for i in range(self._tensor.ndim)]

    # tensor access
    @property
    def tensor(self):
        return self._tensor

    @tensor.setter
    def tensor(self, value):
        self._tensor = np.asarray(value)

    def set_tensor(self, tensor):
        self._tensor = np.asarray(tensor)

    @property
    def shape(self):
        return self._tensor.shape

    # edges
    def get_edge(self, key):
        if isinstance(key, str):
            for e in self.edges:
                if e.name == key:
                    return e
            raise ValueError(f"no edge named {key}")
        return self.edges[key]

    def __getitem__(self, key):
        return self.get_edge(key)

    def add_edge(self, edge, axis, override=False):
        self.edges[axis] = edge

    def get_all_edges(self):
        return list(self.edges)

    def get_all_dangling(self):
        return {e for e in self.edges if e.is_dangling()}

    def get_all_nondangling(self):
        return {e for e in self.edges if not e.is_dangling()}

    def has_nondangling_edge(self):
        return any(not e.is_dangling() for e in self.edges)

    def reorder_edges(self, edge_order):
        if set(map(id, edge_order)) != set(map(id, self.edges)) or \
                len(edge_order) != len(self.edges):
            raise ValueError("edge_order is not a permutation of the edges")
        perm = [next(i for i, e in enumerate(self.edges) if e is o)
                for o in edge_order]
        self._tensor = np.transpose(self._tensor, perm)
        old_edges = self.edges
        self.edges = list(edge_order)
        for new_axis, old_axis in enumerate(perm):
            e = old_edges[old_axis]
            if e.node1 is self and e.axis1 == old_axis:
                e.axis1 = new_axis
            elif e.node2 is self and e.axis2 == old_axis:
                e.axis2 = new_axis
        return self

    def fresh_edges(self):
        if len(self.axis_names) != self._tensor.ndim:
            self.axis_names = [None] * self._tensor.ndim
        self.edges = [Edge(self, i, name=self.axis_names[i])
                      for i in range(self._tensor.ndim)]

    def copy(self, conjugate=False):
        t = np.conj(self._tensor) if conjugate else self._tensor
        return Node(t, name=self.name, axis_names=self.axis_names)

    def __str__(self):
        return self.name

    def __repr__(self):
        return f"Node({self.name}, shape={self.shape})"


def connect(edge1, edge2, name=None):
    if edge1 is edge2:
        raise ValueError("Cannot connect an edge to itself.")
    if not edge1.is_dangling() or not edge2.is_dangling():
        raise ValueError("Both edges must be dangling.")
    if edge1.dimension != edge2.dimension:
        raise ValueError("Edge dimensions do not match.")
    new = Edge(node1=edge1.node1, axis1=edge1.axis1, name=name,
               node2=edge2.node1, axis2=edge2.axis1)
    edge1.node1.edges[edge1.axis1] = new
    edge2.node1.edges[edge2.axis1] = new
    return new


def get_shared_edges(node1, node2):
    out = set()
    for e in node1.edges:
        if not e.is_dangling() and (
                (e.node1 is node1 and e.node2 is node2) or
                (e.node1 is node2 and e.node2 is node1)):
            out.add(e)
    return out


def _rewire(result, sources_and_skip):
    """Give ``result`` the free edges of the sources, in order."""
    edges = []
    for node, skip in sources_and_skip:
        for axis, e in enumerate(node.edges):
            if axis in skip:
                continue
            edges.append((e, node, axis))
    for new_axis, (e, node, axis) in enumerate(edges):
        e.update_axis(axis, node, new_axis, result)
        result.edges[new_axis] = e
    # Consumed nodes keep their tensors and get fresh dangling edges, so a
    # node (e.g. one gate) can be contracted again later.
    for node, _ in sources_and_skip:
        node.fresh_edges()
    return result


def contract_between(node1, node2, name=None, allow_outer_product=False,
                     output_edge_order=None):
    if node1 is node2:
        raise ValueError("contract_between of a node with itself is unsupported")
    shared = list(get_shared_edges(node1, node2))
    if not shared and not allow_outer_product:
        raise ValueError("No edges found between nodes.")
    axes1, axes2 = [], []
    for e in shared:
        if e.node1 is node1:
            axes1.append(e.axis1)
            axes2.append(e.axis2)
        else:
            axes1.append(e.axis2)
            axes2.append(e.axis1)
    t = np.tensordot(node1.tensor, node2.tensor, axes=(axes1, axes2))
    new = Node(t, name=name)
    _rewire(new, [(node1, set(axes1)), (node2, set(axes2))])
    if output_edge_order is not None:
        new.reorder_edges(output_edge_order)
    return new


def contract(edge, name=None):
    if edge.is_dangling():
        raise ValueError("Attempting to contract a dangling edge.")
    n1, n2 = edge.node1, edge.node2
    if n1 is n2:
        raise ValueError("Trace edges are unsupported by this restatement.")
    t = np.tensordot(n1.tensor, n2.tensor, axes=([edge.axis1], [edge.axis2]))
    new = Node(t, name=name)
    _rewire(new, [(n1, {edge.axis1}), (n2, {edge.axis2})])
    return new


def flatten_edges_between(node1, node2):
    shared = list(get_shared_edges(node1, node2))
    if not shared:
        return None
    if len(shared) == 1:
        return shared[0]
    dims = [e.dimension for e in shared]
    for node in (node1, node2):
        axes = [e.axis1 if e.node1 is node else e.axis2 for e in shared]
        keep = [i for i in range(node.tensor.ndim) if i not in axes]
        perm = keep + axes
        t = np.transpose(node.tensor, perm)
        t = np.reshape(t, [node.tensor.shape[i] for i in keep] + [int(np.prod(dims))])
        old_edges = node.edges
        node._tensor = t
        node.axis_names = [node.axis_names[i] for i in keep] + [None]
        node.edges = [old_edges[i] for i in keep] + [None]
        for new_axis, old_axis in enumerate(keep):
            old_edges[old_axis].update_axis(old_axis, node, new_axis, node)
    a1 = node1.tensor.ndim - 1
    a2 = node2.tensor.ndim - 1
    new = Edge(node1=node1, axis1=a1, node2=node2, axis2=a2)
    node1.edges[a1] = new
    node2.edges[a2] = new
    return new


def svd_decomposition(tensor, split_axis, max_singular_values=None,
                      max_truncation_error=None):
    left_dims = tensor.shape[:split_axis]
    right_dims = tensor.shape[split_axis:]
    mat = np.reshape(tensor, [int(np.prod(left_dims)), int(np.prod(right_dims))])
    u, s, vh = np.linalg.svd(mat, full_matrices=False)
    if max_singular_values is None:
        max_singular_values = np.size(s)
    if max_truncation_error is not None:
        trunc_errs = np.sqrt(np.cumsum(np.square(s[::-1])))
        num_err = np.count_nonzero(trunc_errs > max_truncation_error)
    else:
        num_err = max_singular_values
    keep = min(max_singular_values, num_err)
    s = s.astype(mat.dtype)
    s_rest = s[keep:]
    s = s[:keep]
    u = u[:, :keep]
    vh = vh[:keep, :]
    dim_s = s.shape[0]
    u = np.reshape(u, list(left_dims) + [dim_s])
    vh = np.reshape(vh, [dim_s] + list(right_dims))
    return u, s, vh, s_rest


def _attach_split(node, left_edges, right_edges, left_node, right_node):
    nl = len(left_edges)
    for i, e in enumerate(left_edges):
        left_node.edges[i] = e
        e.update_axis(i, node, i, left_node)
    for i, e in enumerate(right_edges):
        right_node.edges[i + 1] = e
        e.update_axis(i + nl, node, i + 1, right_node)


def split_node(node, left_edges, right_edges, max_singular_values=None,
               max_truncation_err=None, left_name=None, right_name=None,
               edge_name=None):
    node.reorder_edges(list(left_edges) + list(right_edges))
    u, s, vh, rest = svd_decomposition(node.tensor, len(left_edges),
                                       max_singular_values, max_truncation_err)
    sq = np.sqrt(s)
    u_s = u * sq
    vh_s = np.reshape(sq, [sq.shape[0]] + [1] * (vh.ndim - 1)) * vh
    left_node = Node(u_s, name=left_name)
    right_node = Node(vh_s, name=right_name)
    _attach_split(node, left_edges, right_edges, left_node, right_node)
    node.fresh_edges()
    connect(left_node.edges[-1], right_node.edges[0], name=edge_name)
    return left_node, right_node, rest


def split_node_full_svd(node, left_edges, right_edges, max_singular_values=None,
                        max_truncation_err=None, left_name=None,
                        middle_name=None, right_name=None, left_edge_name=None,
                        right_edge_name=None):
    node.reorder_edges(list(left_edges) + list(right_edges))
    u, s, vh, rest = svd_decomposition(node.tensor, len(left_edges),
                                       max_singular_values, max_truncation_err)
    left_node = Node(u, name=left_name)
    s_node = Node(np.diag(s), name=middle_name)
    right_node = Node(vh, name=right_name)
    _attach_split(node, left_edges, right_edges, left_node, right_node)
    node.fresh_edges()
    connect(left_node.edges[-1], s_node.edges[0], name=left_edge_name)
    connect(s_node.edges[1], right_node.edges[0], name=right_edge_name)
    return left_node, s_node, right_node, rest


def copy(nodes, conjugate=False):
    nodes = list(nodes)
    node_dict = {n: n.copy(conjugate) for n in nodes}
    edge_dict = {}
    for n in nodes:
        for axis, e in enumerate(n.edges):
            if e in edge_dict:
                continue
            if e.is_dangling():
                ne = Edge(node_dict[n], axis, name=e.name)
                node_dict[n].edges[axis] = ne
            elif e.node1 in node_dict and e.node2 in node_dict:
                ne = Edge(node_dict[e.node1], e.axis1, name=e.name,
                          node2=node_dict[e.node2], axis2=e.axis2)
                node_dict[e.node1].edges[e.axis1] = ne
                node_dict[e.node2].edges[e.axis2] = ne
            else:
                ne = Edge(node_dict[n], axis, name=e.name)
                node_dict[n].edges[axis] = ne
            edge_dict[e] = ne
    return node_dict, edge_dict


def check_connected(nodes):
    nodes = list(nodes)
    if not nodes:
        return
    members = set(map(id, nodes))
    seen = {id(nodes[0])}
    stack = [nodes[0]]
    while stack:
        cur = stack.pop()
        for e in cur.edges:
            if e.is_dangling():
                continue
            for other in (e.node1, e.node2):
                if id(other) in members and id(other) not in seen:
                    seen.add(id(other))
                    stack.append(other)
    if seen != members:
        raise ValueError("Non-connected graph")
