"""The benchmark's end-to-end loop moves every step's state through pinned
host memory and overlaps the downloads of one step with the uploads of the
next (bench.host_round_trips).  Here that loop, with chunks small enough that
every leaf is split, must leave the host buffers holding exactly what the
same number of plain rk4_step calls on device tensors gives
(JAX_BSSN/evolution/time_evolve.py:144-217): a Teukolsky wave with Sommerfeld
faces, three steps, bit for bit on every leaf.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_pipelined_round_trips_equal_plain_steps(cuda, native):
    import bench
    import jax_bssn_gb300 as pkg
    from jax_bssn_gb300.evolution.time_evolve import rk4_step
    from jax_bssn_gb300.initial_data import teukolsky_config
    state, params = teukolsky_config(n=24)
    leaves = [np.ascontiguousarray(f) for f in state]
    host = [torch.from_numpy(f.copy()).pin_memory() for f in leaves]
    dev = [h.to("cuda") for h in host]
    stream = torch.cuda.current_stream()

    def step(d):
        return list(rk4_step(pkg.BSSNVariables(*d), params))

    bench.host_round_trips(step, dev, host, 3, stream, chunk_bytes=40000)
    torch.cuda.synchronize()
    want = [torch.from_numpy(f.copy()).to("cuda") for f in leaves]
    for _ in range(3):
        want = step(want)
    for leaf, h, w in zip(pkg.BSSNVariables._fields, host, want):
        np.testing.assert_array_equal(h.numpy(), w.cpu().numpy(), err_msg=leaf)
