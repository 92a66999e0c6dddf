"""Python host mirror of the learned-proposal C ABI (include/lrt_proposal.h).

The proposal state lives in a ``lrt.Scene``'s context: triples are collected
from that scene's plain renders, the network trains on the GPU, and
``scene.set_tuning("proposal", 1)`` switches the scene's renders to the
proposal kernel.  No CPU fallback.
"""
import ctypes as C

import numpy as np

from . import lrt

N_PARAMS, N_FEATURES = 1633, 16
OFF_W1, OFF_B1, OFF_W2, OFF_B2, OFF_W3, OFF_B3 = 0, 512, 544, 1568, 1600, 1632

_bound = False


def _lib():
    global _bound
    L = lrt.lib()
    if not _bound:
        P, U32, U64, VP = C.c_void_p, C.c_uint32, C.c_uint64, C.c_void_p
        I = C.c_int
        sig = {
            "lrt_proposal_set_weights": (I, [P, VP]),
            "lrt_proposal_get_weights": (I, [P, VP]),
            "lrt_proposal_collect": (I, [P, VP, U32, U64, C.POINTER(U64)]),
            "lrt_proposal_set_triples": (I, [P, VP, VP, U64]),
            "lrt_proposal_clear": (I, [P]),
            "lrt_proposal_get_triples": (I, [P, U64, U64, VP, VP]),
            "lrt_proposal_train": (I, [P, U32, U32, U32, C.c_float, U32, VP]),
            "lrt_proposal_gradient": (I, [P, U32, VP, VP]),
            "lrt_proposal_infer": (I, [P, U64, U64, VP]),
            "lrt_proposal_infer_ex": (I, [P, U64, U64, VP, I, VP]),
            "lrt_proposal_stats": (I, [P, VP]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _bound = True
    return L


def init_weights(seed=7):
    """He-uniform hidden layers, small output layer, zero biases (numpy, seeded)."""
    rng = np.random.default_rng(seed)
    w = np.zeros(N_PARAMS, np.float32)
    w[OFF_W1:OFF_B1] = rng.uniform(-1, 1, 512) * np.sqrt(6.0 / 16)
    w[OFF_W2:OFF_B2] = rng.uniform(-1, 1, 1024) * np.sqrt(6.0 / 32)
    w[OFF_W3:OFF_B3] = rng.uniform(-1, 1, 32) * np.sqrt(1.0 / 32)
    w[OFF_B3] = 0.5
    return w


def _chk(scene, s):
    if s != 0:
        raise lrt.LrtError(s, lrt.lib().lrt_last_error(scene._ctx).decode())


def set_weights(scene, w):
    w = np.ascontiguousarray(w, np.float32)
    assert w.size == N_PARAMS
    _chk(scene, _lib().lrt_proposal_set_weights(scene._ctx, lrt._ptr(w)))


def get_weights(scene):
    w = np.zeros(N_PARAMS, np.float32)
    _chk(scene, _lib().lrt_proposal_get_weights(scene._ctx, lrt._ptr(w)))
    return w


def collect(scene, views, capacity):
    va = lrt.make_views(views)
    n = C.c_uint64()
    _chk(scene, _lib().lrt_proposal_collect(scene._ctx, C.cast(va, C.c_void_p), len(views), capacity, C.byref(n)))
    return n.value


def clear(scene):
    _chk(scene, _lib().lrt_proposal_clear(scene._ctx))


def set_triples(scene, features, targets):
    f = np.ascontiguousarray(features, np.float32).reshape(-1, N_FEATURES)
    t = np.ascontiguousarray(targets, np.float32)
    _chk(scene, _lib().lrt_proposal_set_triples(scene._ctx, lrt._ptr(f), lrt._ptr(t), t.size))


def get_triples(scene, first, n):
    f = np.zeros((n, N_FEATURES), np.float32)
    t = np.zeros(n, np.float32)
    _chk(scene, _lib().lrt_proposal_get_triples(scene._ctx, first, n, lrt._ptr(f), lrt._ptr(t)))
    return f, t


def train(scene, steps, batch=8192, lr=1e-3, seed=7, first_step=0):
    losses = np.zeros(steps, np.float32)
    _chk(scene, _lib().lrt_proposal_train(scene._ctx, first_step, steps, batch, lr, seed, lrt._ptr(losses)))
    return losses


def gradient(scene, n):
    g = np.zeros(N_PARAMS, np.float32)
    loss = np.zeros(1, np.float32)
    _chk(scene, _lib().lrt_proposal_gradient(scene._ctx, n, lrt._ptr(g), lrt._ptr(loss)))
    return float(loss[0]), g


ENGINE_MMA = 0
ENGINE_TCGEN05 = 1


def infer(scene, first, n, engine=None, timed=False):
    """Network outputs for triples [first, first + n); `engine` picks the
    tensor-core path (ENGINE_MMA or ENGINE_TCGEN05).  With timed=True returns
    (outputs, kernel milliseconds)."""
    out = np.zeros(n, np.float32)
    if engine is None and not timed:
        _chk(scene, _lib().lrt_proposal_infer(scene._ctx, first, n, lrt._ptr(out)))
        return out
    ms = np.zeros(1, np.float32)
    _chk(scene, _lib().lrt_proposal_infer_ex(scene._ctx, first, n, lrt._ptr(out),
                                             ENGINE_MMA if engine is None else engine, lrt._ptr(ms)))
    return (out, float(ms[0])) if timed else out


def stats(scene):
    out = np.zeros(4, np.uint64)
    _chk(scene, _lib().lrt_proposal_stats(scene._ctx, lrt._ptr(out)))
    return {"proposals": int(out[0]), "jumps": int(out[1]), "jump_hits": int(out[2]), "steps_skipped": int(out[3])}
