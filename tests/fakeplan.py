"""Duck-typed stand-ins for the reference's plan objects, built from a
Program, so the plugin's reference-facing entry points can be exercised where
the reference itself is absent.  They expose exactly what the plugin reads:
``plan.tree.iterate_postorder()`` nodes (``is_leaf``, ``tensor_index``,
``left_edge_map``, ``right_edge_map``), ``plan.network.index_list(t)``,
``plan.network[t]`` (``shape``, ``build(factory)``) and
``plan.groups_to_slice``."""
from tensororder_gb300.program import join_edges


class FakeTensor:
    def __init__(self, leaf):
        self._leaf = leaf
        self.shape = (2,) * leaf.rank

    def build(self, factory):
        out = factory(self.shape)
        out[...] = self._leaf.parent()
        return out


class FakeNode:
    def __init__(self, is_leaf, tensor_index=None, lmap=None, rmap=None):
        self.is_leaf = is_leaf
        self.tensor_index = tensor_index
        self.left_edge_map = lmap
        self.right_edge_map = rmap


class FakeTree:
    def __init__(self, nodes):
        self._nodes = nodes

    def iterate_postorder(self):
        return iter(self._nodes)


class FakeNetwork:
    def __init__(self, leaves):
        self._leaves = leaves

    def index_list(self, t):
        return list(self._leaves[t].axes)

    def __getitem__(self, t):
        return FakeTensor(self._leaves[t])


class FakePlan:
    def __init__(self, program):
        nodes = []
        stack = []
        for t in program.postorder:
            if t >= 0:
                nodes.append(FakeNode(True, t))
                stack.append(list(program.leaves[t].axes))
            else:
                r = stack.pop()
                l = stack.pop()
                lmap, rmap, free = join_edges(l, r)
                nodes.append(FakeNode(False, lmap=lmap, rmap=rmap))
                stack.append(free)
        self.tree = FakeTree(nodes)
        self.network = FakeNetwork(program.leaves)
        self.groups_to_slice = [set(g) for g in program.slice_groups]
