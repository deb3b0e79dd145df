"""Drop-in for the reference's Python binding module ``cmake_example``.

The reference builds a pybind11 module named ``cmake_example`` exposing
``BNSL_PCStable`` and ``BNL_PCStable`` with positional arguments
(python/api_main.cpp:9-12) and drives them from python/pyfastpgm.py:37-90.  This
module exposes the same functions and argument order over the engine's C ABI::

    from fastpgm_gb300 import cmake_example as fastpgm
    fastpgm.BNSL_PCStable(verbose, num_threads, group_size, alpha, ref_net_file,
                          dpath + train_set_file, save_struct)

Where the reference prints an error and exits the process, this raises
``fastpgm_gb300.FpgmError``.  The reference's inference jobs (BNEI_JT, C_PCStable_JT)
are not part of this engine.
"""
from . import bnl_pcstable as _bnl
from . import bnsl_pcstable as _bnsl


def BNSL_PCStable(verbose, n_threads, group_size, alpha, ref_net, train_set, save_struct):
    """PC-stable structure learning on a CSV; writes ``train_set + "_struct"`` when save_struct
    and prints the SHD against ``ref_net`` (a BIF file) when one is given."""
    _bnsl(int(verbose), int(n_threads), int(group_size), float(alpha), str(ref_net), str(train_set),
          bool(save_struct))


def BNL_PCStable(verbose, n_threads, group_size, alpha, ref_net, train_set, save_struct, save_param):
    """BNSL_PCStable followed by maximum-likelihood parameters (Laplace alpha 1) for the learned
    graph; writes ``train_set + "_param"`` when save_param."""
    _bnl(int(verbose), int(n_threads), int(group_size), float(alpha), str(ref_net), str(train_set),
         bool(save_struct), bool(save_param))
