"""Checkpoint and resume (flowket.callbacks.checkpoint drop-in).

``save_optimizer_weights`` / ``load_optimizer_weights`` restate
callbacks/checkpoint.py:9-26 (optimiser state with the epoch and batch in
``<filepath>_optimizer.pkl``); ``save_weights`` / ``load_weights`` hold a
machine's flat parameter vector with its layout; ``CheckpointByTime``
restates callbacks/checkpoint.py:29-73 for a step loop: call
``on_batch_end`` after each step, ``on_epoch_begin`` and ``on_train_end``
as Keras would. Tensors are stored on the host.
"""
import os
import pickle
import time

import torch


def _to_host(x):
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().clone()
    if isinstance(x, dict):
        return {k: _to_host(v) for k, v in x.items()}
    return x


def save_weights(machine, filepath):
    layout = [(name, tuple(shape), off) for name, shape, off in getattr(machine, "layout", [])]
    torch.save({"params": _to_host(machine.params), "layout": layout}, filepath)


def load_weights(machine, filepath):
    state = torch.load(filepath, map_location="cpu")
    layout = [(name, tuple(shape), off) for name, shape, off in getattr(machine, "layout", [])]
    if layout and state["layout"] and state["layout"] != layout:
        raise ValueError("checkpoint layout does not match the machine")
    if state["params"].numel() != machine.params.numel():
        raise ValueError("checkpoint holds %d parameters, the machine %d" % (state["params"].numel(),
                                                                          machine.params.numel()))
    machine.params.copy_(state["params"].to(machine.params.device))
    machine.params_updated()


def save_optimizer_weights(optimizer, filepath, epoch, batch):
    with open(filepath + "_optimizer.pkl", "wb") as f:
        pickle.dump((_to_host(optimizer.state_dict()), epoch, batch), f)


def load_optimizer_weights(optimizer, filepath):
    filepath += "_optimizer.pkl"
    if not os.path.exists(filepath):
        return None
    with open(filepath, "rb") as f:
        state, epoch, batch = pickle.load(f)
    optimizer.load_state_dict(state)
    return epoch, batch


def save_sampler_state(sampler, filepath):
    """The sampler's draw position (Philox seed and offset, or the chains and
    their sweep counter) in ``<filepath>_sampler.pt``, so that a resumed run
    draws what the uninterrupted one would have. The reference keeps no
    sampler state (numpy's global RNG); this makes the resume exact."""
    torch.save(_to_host(sampler.state_dict()), filepath + "_sampler.pt")


def load_sampler_state(sampler, filepath):
    filepath += "_sampler.pt"
    if not os.path.exists(filepath):
        return False
    sampler.load_state_dict(torch.load(filepath, map_location="cpu"))
    return True


class CheckpointByTime:
    """Save the machine (and optimiser state) every ``save_frequency_in_minutes``
    and at the end of training; ``filepath`` may hold format fields filled
    from the logs."""

    def __init__(self, machine, optimizer, filepath, save_frequency_in_minutes=30, save_weights_only=True,
                 sampler=None):
        self.machine = machine
        self.optimizer = optimizer
        self.sampler = sampler
        self.filepath = filepath
        self.save_weights_only = save_weights_only
        self.save_frequency_in_minutes = save_frequency_in_minutes
        self.last_save_time = time.time()
        self.current_epoch = 0

    def _save(self, logs, batch):
        filepath = self.filepath.format(**(logs or {}))
        save_weights(self.machine, filepath)
        if self.optimizer is not None:
            save_optimizer_weights(self.optimizer, filepath, self.current_epoch, batch)
        if self.sampler is not None:
            save_sampler_state(self.sampler, filepath)
        self.last_save_time = time.time()

    def on_batch_end(self, batch, logs=None):
        if time.time() - self.last_save_time < self.save_frequency_in_minutes * 60:
            return
        self._save(logs, batch)

    def on_epoch_begin(self, epoch, logs=None):
        self.current_epoch = epoch

    def on_train_end(self, logs=None):
        self.current_epoch += 1
        self._save(logs, 0)
