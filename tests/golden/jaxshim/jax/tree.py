"""``jax.tree`` stand-in: structural map over tuples, lists, dicts and NamedTuples."""


def _is_namedtuple(value):
    return isinstance(value, tuple) and hasattr(value, "_fields")


def map(f, tree, *rest, is_leaf=None):
    if is_leaf is not None and is_leaf(tree):
        return f(tree, *rest)
    if _is_namedtuple(tree):
        return type(tree)(*(map(f, *items, is_leaf=is_leaf) for items in zip(tree, *rest)))
    if isinstance(tree, (tuple, list)):
        return type(tree)(map(f, *items, is_leaf=is_leaf) for items in zip(tree, *rest))
    if isinstance(tree, dict):
        return {key: map(f, tree[key], *(r[key] for r in rest), is_leaf=is_leaf) for key in tree}
    if tree is None:
        return None
    return f(tree, *rest)


def leaves(tree):
    out = []
    map(lambda leaf: out.append(leaf), tree)
    return out
