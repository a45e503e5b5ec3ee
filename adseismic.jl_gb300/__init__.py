"""adseismic_gb300 -- GB300 (sm_103a) implementation of ADSeismic's time-stepping
hot path: acoustic and elastic one-step operators, their adjoints, source
injection, receiver sampling, misfit and checkpointed multi-shot gradients.

All compute runs in libadseismic_gb300.so (C ABI: include/adseismic_gb300.h).
This package mirrors the reference's Julia interface on top of it.
"""
from . import _lib
from ._lib import AdsError, ADS_F32, ADS_F64, ADS_VARIANT_U, ADS_VARIANT_W, lib
from .build import build_library, LIB_PATH
from .acoustic import (AcousticMisfit, AcousticOneStep, AcousticPlan, AcousticPropagator,
                       AcousticPropagatorParams, AcousticPropagatorSolver, AcousticReceiver,
                       AcousticSource, SimulatedObservation, acoustic_one_step,
                       acoustic_one_step_grad, compute_forward_GPU, compute_loss_and_grads_GPU,
                       dropin_loss_and_grad, step_variant)
from .acoustic import compute_PML_Params as compute_acoustic_PML_Params
from .elastic import (ElasticMisfit, ElasticPlan, ElasticPropagator, ElasticPropagatorParams,
                      ElasticPropagatorSolver, ElasticReceiver, ElasticSource,
                      elastic_one_step, elastic_one_step_grad)
from .elastic import SimulatedObservation as ElasticSimulatedObservation
from .elastic import compute_PML_Params as compute_elastic_PML_Params
from .io import (load_acoustic_model, load_acoustic_receiver, load_acoustic_source,
                 load_elastic_model, load_elastic_receiver, load_elastic_source, load_params)
from .optim import LBFGS, fwi_lbfgs, source_lbfgs, source_objective, wavelet_lbfgs
from .utils import (Gauss, Ricker, add_initial_model, compute_lame_parameters,
                    compute_properties, compute_properties_grad, gradtest,
                    folded_layer_model, gaussian_smooth, layered_gaussian_model,
                    ricker_width_samples, variable_source, variable_source_grad)


def version() -> str:
    return lib().ads_version().decode()


def launch_count() -> int:
    """Number of this library's kernels launched by the process so far."""
    return int(lib().ads_launch_count())
