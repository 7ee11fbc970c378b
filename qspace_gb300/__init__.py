"""qspace_gb300 -- GB300-native block-sparse symmetric tensor contraction.

A drop-in for QSpace's contractQS / permuteQS numerical core (block-sparse
contraction with exact label bookkeeping) with a plain FP64 path and a
split-precision BF16 tensor-core path; eigQS / svdQS / orthoQS over block
eig/SVD on the GPU; a serving loop.
The numerical work runs in libqsgpu.so (CUDA for sm_103a) behind the C-ABI
of include/qsgpu.h.
"""
from .qspace import (QSpace, Tensor, Context, contractQS, contract_batch, contract_itags, permuteQS, default_context, upload,
                     contract_dev, permute_dev)
from .linalg import eigQS, orthoQS, svdQS

__all__ = ["QSpace", "Tensor", "Context", "contractQS", "contract_batch", "contract_itags", "permuteQS", "default_context",
           "upload", "contract_dev", "permute_dev", "eigQS", "svdQS", "orthoQS"]
