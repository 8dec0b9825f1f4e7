"""qsft_gb300 -- the q-SFT hot path (sparse q-ary Fourier transform) on one GB300.

Drop-in for the reference API of basics-lab/qsft:

    from qsft_gb300 import QSFT, get_random_subsampled_signal, get_reed_solomon_dec

    signal = get_random_subsampled_signal(n=..., q=..., sparsity=..., a_min=..., a_max=...,
                                          noise_sd=..., query_args=query_args)
    result = QSFT(num_subsample=..., num_repeat=..., b=..., reconstruct_method_source="identity",
                  reconstruct_method_channel="nso").transform(signal, report=True)

Every step of the path (coset evaluation, GWHT, noise, singleton detection,
peeling) runs as CUDA kernels of ``lib/libqsft_gb300.so`` (C ABI in
``include/qsft_gb300.h``); there is no CPU fallback.  Batched and continuous
serving: ``qsft_gb300.serve`` (packed batches, pipelined streams) and
``qsft_gb300.server`` (arrivals over time, admission by device footprint);
several GPUs as replicas: ``qsft_gb300.replicas``.
"""
from .engine import Batch, JobSpec, workspace_bytes
from .input_signal_subsampled import Signal, SubsampledSignal
from .qsft import QSFT
from .query import get_D, get_Ms, get_Ms_and_Ds, get_reed_solomon_dec
from .reed_solomon import ReedSolomon
from .synthetic_signal import SyntheticSubsampledSignal, generate_signal_w, get_random_subsampled_signal
from . import replicas, serve, server, utils

__all__ = [
    "QSFT", "Signal", "SubsampledSignal", "SyntheticSubsampledSignal", "get_random_subsampled_signal",
    "generate_signal_w", "get_Ms_and_Ds", "get_Ms", "get_D", "get_reed_solomon_dec", "ReedSolomon", "Batch",
    "JobSpec", "workspace_bytes", "utils", "serve", "server", "replicas",
]
