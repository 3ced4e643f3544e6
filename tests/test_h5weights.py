"""The HDF5 reader on the reference's own Keras weight files
(experiments/weights/*.h5: depth-10, 32-channel, weight-normalised
ConvNetAutoregressive2D for the 12x12 Ising models). Host only; skipped
where those files are not present."""
import os

import numpy as np
import pytest

# directory holding the reference's experiments/weights/*.h5 files (read in
# place, never copied); the tests are skipped when it is not set
REF_WEIGHTS = os.environ.get("FLOWKET_REFERENCE_WEIGHTS")


def _path(name):
    if not REF_WEIGHTS:
        pytest.skip("FLOWKET_REFERENCE_WEIGHTS is not set")
    p = os.path.join(REF_WEIGHTS, name)
    if not os.path.exists(p):
        pytest.skip("reference weight files not present")
    return p


def test_reader_finds_every_layer():
    from flowket_gb300.h5weights import read_keras_weights
    layers = read_keras_weights(_path("ising_3.h5"))
    assert len(layers) == 91  # 18 causal convs x 5 weight-normalised convs + the output conv
    from flowket_gb300.h5weights import _creation_order
    layers = _creation_order(layers)
    shapes = [tuple(ws[0][1].shape) for _, ws in layers]
    # per causal conv: v 3x3, h 1x3, x 1x1 -> F/2, y 1x1 -> F/2, c 3x3
    assert shapes[:5] == [(3, 3, 1, 32), (1, 3, 1, 32), (1, 1, 32, 16), (1, 1, 32, 16), (3, 3, 32, 32)]
    assert shapes[5:10] == [(3, 3, 32, 32), (1, 3, 32, 32), (1, 1, 32, 16), (1, 1, 32, 16), (3, 3, 32, 32)]
    assert shapes[-1] == (1, 1, 32, 4)
    assert [n.split("/")[-1] for n, _ in layers[0][1]] == ["kernel:0", "bias:0", "g:0"]
    assert [n.split("/")[-1] for n, _ in layers[-1][1]] == ["kernel:0", "bias:0"]
    for _, ws in layers:
        for _, a in ws:
            assert a.dtype == np.float32 and np.all(np.isfinite(a))


def test_flat_vector_matches_the_machine_layout_and_oracle():
    """The converted vector fills every parameter of the depth-10 layout once,
    and the oracle's network built from it is a normalised AR model."""
    import torch
    from flowket_gb300.h5weights import keras_weights_to_flat, read_keras_weights
    from flowket_gb300.machines import ar2d_param_layout
    from oracle import ar2d
    layout, n = ar2d_param_layout(10, 32, True)
    flat = keras_weights_to_flat(read_keras_weights(_path("ising_2.h5")), layout)
    assert flat.size == n
    params = {name: torch.from_numpy(flat[off:off + int(np.prod(shape))].reshape(shape)).double()
              for name, shape, off in layout}
    # g is the log of each output channel's scale (exponential_norm): trained values, not the init's log-norm
    assert not np.allclose(params["cc0.v.g"].numpy(), np.log(np.linalg.norm(params["cc0.v.kernel"].numpy().reshape(-1, 32), axis=0)))
    x = torch.as_tensor(np.random.default_rng(0).choice([-1, 1], size=(2, 12, 12)).astype(np.int8))
    re, im = ar2d.conditional_log_wave_function(params, x, 10, True)
    np.testing.assert_allclose(torch.exp(2 * re).sum(-1).numpy(), 1.0, rtol=1e-12)
    with pytest.raises(ValueError):
        keras_weights_to_flat(read_keras_weights(_path("ising_2.h5")), ar2d_param_layout(8, 32, True)[0])


def test_reader_rejects_what_it_does_not_read(tmp_path):
    from flowket_gb300.h5weights import read_keras_weights
    p = tmp_path / "x.h5"
    p.write_bytes(b"not an hdf5 file at all" * 4)
    with pytest.raises(ValueError):
        read_keras_weights(str(p))
    # an HDF5 signature with a newer superblock version
    p.write_bytes(b"\x89HDF\r\n\x1a\n" + bytes([2]) + bytes(200))
    with pytest.raises(ValueError):
        read_keras_weights(str(p))
