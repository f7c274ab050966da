"""State checkpoints in the reference's pickle layout (util_op.py:976-1014):
{'fields': {name: ndarray}, 'weights': {name: [ndarray, ...]}}, so reference
checkpoints load as initial states and the engine's load in the reference."""
import pickle

import numpy as np
import torch


def checkpoint_save(state, path):
    """util_op.py:976-989."""
    s = {
        "fields": {k: (v.detach().cpu().numpy() if isinstance(v, torch.Tensor)
                       else np.array(v)) for k, v in state.fields.items()},
        "weights": {k: [np.array(w) for w in ws]
                    for k, ws in state.weights.items()},
    }
    with open(path, "wb") as f:
        pickle.dump(s, f)


def checkpoint_load(state, path, fields_to_load=None, weights_to_load=None,
                    skip_missing=True, device=None, dtype=torch.float64):
    """util_op.py:992-1014; fields go to `device` as torch tensors when given
    (numpy arrays otherwise, converted by Problem.init_missing)."""
    with open(path, "rb") as f:
        try:
            s = pickle.load(f)
        except (pickle.UnpicklingError, EOFError, AttributeError,
                ImportError, IndexError, TypeError, ValueError) as e:
            raise ValueError("corrupt checkpoint %s: %s: %s"
                             % (path, type(e).__name__, e)) from e
    if not isinstance(s, dict):
        raise ValueError("checkpoint %s holds %s, not the {'fields', "
                         "'weights'} dict" % (path, type(s).__name__))
    fields = s.get("fields", None)
    if fields is not None:
        for k in (fields.keys() if fields_to_load is None else fields_to_load):
            if k not in fields:
                if not skip_missing:
                    raise RuntimeError("Missing field {}".format(k))
                continue
            a = np.asarray(fields[k])
            state.fields[k] = a if device is None else torch.as_tensor(
                a, dtype=dtype, device=device)
    weights = s.get("weights", None)
    if weights is not None:
        for k in (weights.keys() if weights_to_load is None else
                  weights_to_load):
            if k not in weights:
                if not skip_missing:
                    raise RuntimeError("Missing weights {}".format(k))
                continue
            state.weights[k] = weights[k]
