"""GB300-native ApplicationClassification matcher.

A from-scratch sm_103a implementation of the graph-matching pipeline of
porumbes/application_classification (src/ac.hxx, src/main.cu): feature cdist,
row log-softmax normalisers, edge->vertex max messages and mu updates, behind
the C ABI in ``include/acg.h``.  This package is the Python host side:

* :mod:`.graph`   -- the reference's binary/CSV graph formats, seeded generators
* :mod:`.matcher` -- DataGraph / Plan / match over the C ABI
* :mod:`.build`   -- builds ``_build/libacg.so``
"""
from .graph import Graph, gen_er, gen_rmat, plant, fill_edges, workload  # noqa: F401
from ._lib import AcgError  # noqa: F401


def __getattr__(name):  # lazy: importing torch is not needed for I/O or generation
    if name in ("DataGraph", "Plan", "DeviceGraph", "match"):
        from . import matcher

        return getattr(matcher, name)
    raise AttributeError(name)


__version__ = "0.1.0"
