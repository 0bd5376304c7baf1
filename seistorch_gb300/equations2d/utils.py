"""Stencil helpers with seistorch's names (seistorch/equations2d/utils.py)."""
import torch


def diff_using_roll(input, dim=-1, forward=True, padding_value=0):
    """forward: x[i] - x[i-1] (0 at i=0); backward: x[i+1] - x[i] (0 at the
    last index) (utils.py:3-48)."""
    if forward:
        diff = input - torch.roll(input, shifts=1, dims=dim)
        idx = [slice(None)] * input.ndim
        idx[dim] = 0
    else:
        diff = torch.roll(input, shifts=-1, dims=dim) - input
        idx = [slice(None)] * input.ndim
        idx[dim] = -1
    diff[tuple(idx)] = padding_value
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
