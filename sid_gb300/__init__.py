"""sid_gb300: GB300-native (sm_103a) implementation of SID's hot path.

The compute lives in ``libsid.so`` (hand-written CUDA behind the C ABI of
``include/sid.h``); this package mirrors the reference's MATLAB functions on
top of it.  Import does not require a GPU; calling the operators does.
"""
from ._lib import SidError  # noqa: F401
from .nnls import Context, LS_nnls, NQP, fast_nnls, quantile, reg_nnls, update_spatial_component  # noqa: F401
from .nmf import S_update, T_update  # noqa: F401
from .background import compute_std_image, rank_1_factorization  # noqa: F401
from .postproc import ImageRect, SNR_order, merge_filters, read_sensor_movie, rectify_frames  # noqa: F401
from .tiff import read_tiff  # noqa: F401
from .matfile import load_psf, matfile_read  # noqa: F401
from .extract import Extractor, incremental_temporal_update_gpu  # noqa: F401
from .lfm import (  # noqa: F401
    LS_deconv,
    Projector,
    backwardProjectACC_new,
    backwardProjectGPU_new,
    deconvRL,
    forwardProjectACC,
    forwardProjectGPU,
    generate_kernel,
    generate_LFM_library_CPU,
    generate_LFM_library_GPU,
    library_boxes,
    library_kernel_voxels,
    reconstruct_S,
    set_default_method,
    to_device,
    to_numpy,
)

__version__ = "1.0.0"
