"""GB300-native SNICIT sparse-DNN inference engine (sm_103a CUDA behind a C ABI).

The compute path is the CUDA library built in-tree (libsnicit_gb300.so);
this package only binds it.  See include/snicit_gb300.h for the ABI.
"""
from ._lib import MODES, SdnnError, load  # noqa: F401
from .engine import (Engine, coo_to_csr, generate_inputs, generate_inputs_device,  # noqa: F401
                     generate_layer_coo, generate_layer_csr, generate_radixnet_layer_coo,
                     inputs_bin_info, pack_bits, read_inputs_bin, read_inputs_tsv,
                     write_categories_tsv, write_inputs_bin, write_inputs_tsv)
from .sdgc import BF, SNICIT, SNIG, XY  # noqa: F401
from .serving import Server, mlp_inputs, request_stream, sparse_mlp  # noqa: F401
