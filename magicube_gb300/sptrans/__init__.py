"""Drop-in mirror of the reference's ``sptrans`` torch extension ops.

Same module names, function names, argument order and output shapes as the
reference's extension (end2end_eval/sparse_transformer_magicube/src/cuda/
{quantization,deq_sddmm,q_softmax,deq_spmm}.cpp), computed by this library's
sm_103a kernels through its C ABI on torch's current CUDA stream:

    from magicube_gb300.sptrans.quantization import bquantization
    from magicube_gb300.sptrans.deq_sddmm import bsddmm_8b
    from magicube_gb300.sptrans.q_softmax import q_bcsr_softmax
    from magicube_gb300.sptrans.deq_spmm import bspmm_8b

Differences from the reference, all deliberate:
  * integer lanes are two's complement throughout (the reference feeds signed
    quantized data to unsigned .u8/.u4 MMAs, which is only correct for
    non-negative values);
  * inputs are made contiguous before use (the reference reads the raw
    storage of transposed views);
  * arguments are checked and errors raised instead of printed;
  * the softmax's running maximum starts from -inf for every vector lane.
"""
from . import deq_sddmm, deq_spmm, q_softmax, quantization  # noqa: F401
