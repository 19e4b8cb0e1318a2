"""Host-side logic of the optimisers' reference interface (masked_adam.py):
the hyper-parameter checks of VDBAdam and MaskedAdam raise the reference's
ValueError messages before any device work (no GPU needed)."""
import pytest


@pytest.mark.parametrize("kw,msg", [
    ({"lr": -1.0}, "Invalid learning rate: -1.0"),
    ({"eps": -1e-8}, "Invalid epsilon value: -1e-08"),
    ({"betas": (1.0, 0.99)}, "Invalid beta parameter at index 0: 1.0"),
    ({"betas": (0.9, -0.1)}, "Invalid beta parameter at index 1: -0.1"),
])
def test_hparam_checks(kw, msg):
    import torch

    from plenvdb_gb300.masked_adam import MaskedAdam, VDBAdam
    with pytest.raises(ValueError, match=msg.replace("(", r"\(").replace(".", r"\.")):
        MaskedAdam([torch.zeros(3, requires_grad=True)], **kw)
    with pytest.raises(ValueError, match=msg.replace(".", r"\.")):
        VDBAdam([], **kw)


def test_valid_hparams_build_groups():
    import torch

    from plenvdb_gb300.masked_adam import MaskedAdam
    p = torch.zeros(3, requires_grad=True)
    opt = MaskedAdam([p], lr=1e-3, betas=(0.9, 0.99), eps=1e-8)
    g = opt.param_groups[0]
    assert g["lr"] == 1e-3 and g["betas"] == (0.9, 0.99) and g["eps"] == 1e-8
    assert opt.per_lr is None
