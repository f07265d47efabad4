"""CUDA (sm_103a) solvers and formulas: the sqaod.cuda API on libsqaod_gb300.so."""
from . import formulas
from .solvers import (BipartiteGraphAnnealer, BipartiteGraphBFSearcher, DenseGraphAnnealer,
                      DenseGraphBFSearcher, bipartite_graph_annealer, bipartite_graph_bf_searcher,
                      dense_graph_annealer, dense_graph_bf_searcher)
