"""jax.tree_util stand-in: tuples and lists are the only containers."""


def register_pytree_node_class(cls):
    return cls


def tree_map(f, tree, *rest):
    if isinstance(tree, tuple):
        return tuple(tree_map(f, t, *(r[i] for r in rest)) for i, t in enumerate(tree))
    if isinstance(tree, list):
        return [tree_map(f, t, *(r[i] for r in rest)) for i, t in enumerate(tree)]
    return f(tree, *rest)
