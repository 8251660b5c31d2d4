"""The split kernel's bounded waits: a wait that runs out ends the launch
with ATRIP_ERR_TIMEOUT and leaves the context usable.

The test knob split_test_unpublished makes the kernel's producer publish no
tuple at all, so the MMA issuer, the epilogue and the energy warps each wait
on a tuple hand-off barrier that nothing arms.  No bulk copy and no MMA is
ever issued; with a short limit (split_wait_kcycles) the waits give up, the
CTAs release their tensor memory and leave, the host reads the status word
and returns the timeout.  A normal run on the same context then matches the
result from before.
"""
import pytest

from atrip_gb300 import capi, synth

pytestmark = pytest.mark.gpu
NAMES = ("epsi", "epsa", "Tai", "Tabij", "Vabij", "Vijka", "Vabci")


@pytest.mark.parametrize("form,slices,variant", [("split_f16", 2, 2), ("split_bf16", 3, 0),
                                                 ("split_bf16", 2, 2)])
def test_wait_runs_out_then_context_recovers(form, slices, variant):
    d = synth.make_inputs(6, 11, 3)
    with capi.Context(6, 11, 0) as ctx:
        for n in NAMES:
            ctx.upload(n, d[n])
        ctx.set_tuning(split_variant=variant)
        ref = ctx.run(form=form, slices=slices, use_j=False)
        # ~10 ms limit (2e7 SM cycles)
        ctx.set_tuning(split_variant=variant, split_wait_kcycles=20000, split_test_unpublished=1)
        with pytest.raises(capi.AtripError) as err:
            ctx.run(form=form, slices=slices, use_j=False)
        assert err.value.status == capi.ERR_TIMEOUT
        assert "bounded wait" in str(err.value)
        ctx.set_tuning(split_variant=variant)
        again = ctx.run(form=form, slices=slices, use_j=False)
        assert again.energy == ref.energy
        assert again.tuples_done == ref.tuples_done


def test_wait_knobs_are_validated():
    with capi.Context(4, 7, 0) as ctx:
        with pytest.raises(capi.AtripError):
            ctx.set_tuning(split_wait_kcycles=-1)
        with pytest.raises(capi.AtripError):
            ctx.set_tuning(split_test_unpublished=2)
