"""Stencil helpers with seistorch's names (seistorch/equations2d/utils.py)."""
import torch


def diff_using_roll(input, dim=-1, forward=True, padding_value=0):
    """forward: x[i] - x[i-1]; backward: x[i+1] - x[i] (utils.py:3-48).

    The wrapped edge value is replaced by ``padding_value`` only for
    ``dim == 1`` (index 0 / -1 of axis 1) and ``dim == 2`` (index 0 / -1 of
    the LAST axis); any other ``dim`` keeps the roll's wrap, as the
    reference does."""
    edge = 0 if forward else -1
    if forward:
        diff = input - torch.roll(input, shifts=1, dims=dim)
    else:
        diff = torch.roll(input, shifts=-1, dims=dim) - input
    if dim == 1:
        diff[:, edge] = padding_value
    elif dim == 2:
        diff[..., edge] = padding_value
    return diff


def save_boundaries(tensor, NPML=49, N=1):
    """Rows/columns NPML and -(NPML+1) (utils.py:50-69)."""
    top = tensor[:, NPML:NPML + N, :].clone()
    bottom = tensor[:, -N:, :].clone() if NPML == 0 else tensor[:, -(NPML + N):-NPML, :].clone()
    left = tensor[..., NPML:NPML + N].clone()
    right = tensor[..., -N:].clone() if NPML == 0 else tensor[..., -(NPML + N):-NPML].clone()
    return top, bottom, left, right


def restore_boundaries(tensor, memory, NPML=49, N=1, multiple=False):
    """Write the strips of ``save_boundaries`` back (utils.py:71-90)."""
    top, bottom, left, right = memory
    if not multiple:
        tensor[:, NPML:NPML + N, :] = top
    if NPML != 0:
        tensor[:, -(NPML + N):-NPML, :] = bottom
    else:
        tensor[:, -N:, :] = bottom
    tensor[..., NPML:NPML + N] = left
    if NPML != 0:
        tensor[..., -(NPML + N):-NPML] = right
    else:
        tensor[..., :, -N:] = right
    return tensor
