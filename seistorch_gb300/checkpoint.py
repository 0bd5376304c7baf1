"""Per-step boundary-saving autograd of ``WaveCell`` (seistorch/checkpoint_new.py:109-217
for the second-order equations, seistorch/checkpoint.py:108-230 for the others).

With ``boundary_saving`` and ``inversion`` set, the reference's ``WaveCell``
wraps every step in a checkpoint Function (cell.py:71-72).  Its forward runs
the step without autograd and keeps only the one-cell strips of the outputs
(``save_boundaries``).  Its backward walks from the last step down, carrying
the wavefields rebuilt so far:

* the last step's backward hands its own outputs over as the carried state
  (reversed for the second-order equations) and returns no gradient;
* second-order equations (the acoustic family): the next backward (the
  second-to-last step) returns no gradient either; every later one evaluates
  the equation module's ``_time_step_backward`` on the carried state with
  autograd, back-propagates the incoming cotangents through it, carries its
  outputs and returns the gradients of its inputs;
* the other equations (elastic): every backward rebuilds the previous state
  with ``_time_step_backward`` without autograd, carries it, runs
  ``_time_step`` again on it with autograd and back-propagates through that.

This gives the reference's boundary-saving gradient for the same equation
modules -- which is not the pure-autograd gradient, since the reverse step is
not the transpose of the forward step; ``WaveRNN`` uses the exact fused
adjoint instead.  The reference keeps the carried state and a step counter as
class attributes and never resets the counter, so only the first backward of
a process skips the second-to-last step; here both live in a
``ReverseState`` owned by the cell and are reset by the last step's backward,
so every reverse sweep behaves like the reference's first.
"""
import torch

from .equations2d.utils import save_boundaries

_LEAD = 8  # non-tensor arguments ahead of the step's own


class ReverseState:
    """Wavefields rebuilt by the reverse sweep so far, and its step count."""

    def __init__(self):
        self.wavefields = []
        self.count = 0


class _BoundarySavingStep(torch.autograd.Function):
    @staticmethod
    def forward(ctx, state, run_function, back_function, source, is_last, para_counts, second_order, habcs,
                *args):
        ctx.requires = [torch.is_tensor(a) and a.requires_grad for a in args]
        ctx.state, ctx.run, ctx.back, ctx.source = state, run_function, back_function, source
        ctx.second_order, ctx.habcs, ctx.is_last = second_order, habcs, is_last
        with torch.no_grad():
            outputs = run_function(*args, habcs=habcs)
        ctx.models = args[:para_counts]
        ctx.geoms = args[-3:]
        strips = [save_boundaries(o) for o in outputs]
        ctx.nfields = len(outputs)
        ctx.save_for_backward(*[s for st in strips for s in st])
        ctx.lastframe = tuple(o.detach() for o in outputs) if is_last else None
        return outputs

    @staticmethod
    def backward(ctx, *grads):
        st = ctx.state
        nothing = (None,) * (_LEAD + len(ctx.requires))
        if ctx.is_last:
            st.wavefields = list(ctx.lastframe)
            if ctx.second_order:
                st.wavefields.reverse()
            st.count = 0
            return nothing
        st.count += 1
        if st.count == 1 and ctx.second_order:
            return nothing
        saved = ctx.saved_tensors
        strips = [tuple(saved[4 * i:4 * i + 4]) for i in range(ctx.nfields)]

        def leaves(ts):
            return [t.detach().requires_grad_(r) for t, r in zip(ts, ctx.requires)]

        inputs = leaves(list(ctx.models) + list(st.wavefields) + list(ctx.geoms))
        if ctx.second_order:
            with torch.enable_grad():
                outputs = ctx.back(*inputs, strips, ctx.source)
            st.wavefields = [o.detach() for o in outputs]
        else:
            with torch.no_grad():
                rebuilt = ctx.back(*inputs, strips, ctx.source)
            st.wavefields = [o.detach() for o in rebuilt]
            inputs = leaves(list(ctx.models) + list(st.wavefields) + list(ctx.geoms))
            with torch.enable_grad():
                outputs = ctx.run(*inputs, habcs=ctx.habcs)
        pairs = [(o, g) for o, g in zip(outputs, grads) if torch.is_tensor(o) and o.requires_grad]
        if not pairs:
            raise RuntimeError("boundary-saving step: no output of the step requires grad")
        torch.autograd.backward([o for o, _ in pairs], [g for _, g in pairs])
        return (None,) * _LEAD + tuple(t.grad if torch.is_tensor(t) else None for t in inputs)


def boundary_saving_step(state, run_function, back_function, source, is_last, para_counts, second_order, *args,
                         habcs=None):
    """One step of the reference's boundary-saving inversion (cell.py:71-72)."""
    return _BoundarySavingStep.apply(state, run_function, back_function, source, is_last, para_counts,
                                     second_order, habcs, *args)
