"""tcgen05 BF16 convolution kernels of the learned preconditioner vs a plain
PyTorch fp32 reference (conv2d on the same bf16-rounded operands).
Tolerance: relative L2 <= 2e-3 for fp32 outputs (fp32 accumulation in a
different order; bf16 products are exact in fp32)."""
import ctypes

import pytest
import torch
import torch.nn.functional as F

from tests.golden_cases import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def N():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from seistorch_gb300 import _native
    _native.load(build_if_missing=False)
    return _native


def _conv(N, x_nhwc, wt, bias=None, relu=False, mask=None, out_f32=None, out_bf16=None, cstride=None, coff=0):
    n, h, w, cin = x_nhwc.shape
    cout = wt.shape[0]
    c = N.NnConv(n, h, w, cin, cout, N.ptr(x_nhwc), N.ptr(wt), N.ptr(bias), int(relu), N.ptr(mask),
                 mask.shape[-1] if mask is not None else 0, N.ptr(out_bf16), N.ptr(out_f32),
                 cstride or cout, coff)
    N.call("sgb_nn_conv3x3", ctypes.byref(c), N.stream_handle())


def _w9(w):  # torch [cout][cin][3][3] -> [cout][9][cin]
    return w.permute(0, 2, 3, 1).reshape(w.shape[0], 9, w.shape[1]).contiguous()


@pytest.mark.parametrize("n,h,w,cin,cout", [(2, 16, 128, 64, 64), (1, 8, 256, 32, 32), (2, 6, 64, 128, 256),
                                            (1, 5, 128, 96, 128), (1, 4, 512, 64, 32)])
def test_conv_forward_matches_torch(N, n, h, w, cin, cout):
    torch.manual_seed(0)
    dev = torch.device("cuda:0")
    x = torch.randn(n, cin, h, w, device=dev).bfloat16().float()
    wt = (torch.randn(cout, cin, 3, 3, device=dev) / (3 * cin ** 0.5)).bfloat16().float()
    bias = torch.randn(cout, device=dev)
    want = F.relu(F.conv2d(x, wt, bias, padding=1))
    out = torch.empty(n, h, w, cout, device=dev)
    outb = torch.empty(n, h, w, cout, device=dev, dtype=torch.bfloat16)
    _conv(N, x.permute(0, 2, 3, 1).contiguous().bfloat16(), _w9(wt).bfloat16(), bias, True, out_f32=out,
          out_bf16=outb)
    torch.cuda.synchronize()
    got = out.permute(0, 3, 1, 2)
    assert rel_l2(got.cpu().numpy(), want.cpu().numpy()) < 2e-3
    assert rel_l2(outb.float().permute(0, 3, 1, 2).cpu().numpy(), want.cpu().numpy()) < 1e-2


def test_conv_writes_a_channel_slice_and_applies_a_mask(N):
    torch.manual_seed(1)
    dev = torch.device("cuda:0")
    n, h, w, cin, cout = 1, 8, 128, 64, 32
    x = torch.randn(n, cin, h, w, device=dev).bfloat16().float()
    wt = (torch.randn(cout, cin, 3, 3, device=dev) / 24).bfloat16().float()
    mask = torch.randn(n, h, w, cout, device=dev).bfloat16()
    want = F.conv2d(x, wt, padding=1).permute(0, 2, 3, 1) * (mask.float() > 0)
    out = torch.full((n, h, w, 96), 7.0, device=dev)
    _conv(N, x.permute(0, 2, 3, 1).contiguous().bfloat16(), _w9(wt).bfloat16(), mask=mask, out_f32=out,
          cstride=96, coff=32)
    torch.cuda.synchronize()
    assert rel_l2(out[..., 32:64].cpu().numpy(), want.cpu().numpy()) < 2e-3
    assert torch.all(out[..., :32] == 7.0) and torch.all(out[..., 64:] == 7.0)


def test_data_gradient_via_flipped_weights(N):
    torch.manual_seed(2)
    dev = torch.device("cuda:0")
    n, h, w, cin, cout = 2, 8, 128, 32, 64
    x = torch.randn(n, cin, h, w, device=dev, requires_grad=True)
    wt = (torch.randn(cout, cin, 3, 3, device=dev) / 16).bfloat16().float()
    dy = torch.randn(n, cout, h, w, device=dev).bfloat16().float()
    F.conv2d(x, wt, padding=1).backward(dy)
    wflip = wt.flip(2, 3).transpose(0, 1).contiguous()  # [cin][cout][3][3]
    out = torch.empty(n, h, w, cin, device=dev)
    _conv(N, dy.permute(0, 2, 3, 1).contiguous().bfloat16(), _w9(wflip).bfloat16(), out_f32=out)
    torch.cuda.synchronize()
    assert rel_l2(out.permute(0, 3, 1, 2).cpu().numpy(), x.grad.cpu().numpy()) < 2e-3


@pytest.mark.parametrize("n,h,w,cin,cout", [(2, 8, 128, 32, 64), (1, 16, 64, 64, 32), (1, 4, 128, 128, 256)])
def test_weight_gradient_matches_torch(N, n, h, w, cin, cout):
    torch.manual_seed(3)
    dev = torch.device("cuda:0")
    x = torch.randn(n, cin, h, w, device=dev).bfloat16().float()
    wt = torch.zeros(cout, cin, 3, 3, device=dev, requires_grad=True)
    dy = torch.randn(n, cout, h, w, device=dev).bfloat16().float()
    F.conv2d(x, wt, padding=1).backward(dy)
    want = wt.grad.reshape(cout, cin, 9)
    x_nhwc = x.permute(0, 2, 3, 1).contiguous().bfloat16()
    xs = torch.empty(3, n, cin, h, w, device=dev, dtype=torch.bfloat16)
    N.call("sgb_nn_to_chw", n, h, w, cin, cin, 0, N.ptr(x_nhwc), 3, N.ptr(xs), N.stream_handle())
    dy_chw = dy.contiguous().bfloat16()
    dw = torch.zeros(cout, cin, 9, device=dev)
    p = N.NnWgrad(n, h, w, cin, cout, N.ptr(dy_chw), N.PTR3(*[xs[k].data_ptr() for k in range(3)]), N.ptr(dw))
    N.call("sgb_nn_conv3x3_wgrad", ctypes.byref(p), N.stream_handle())
    torch.cuda.synchronize()
    assert rel_l2(dw.cpu().numpy(), want.cpu().numpy()) < 2e-3
    assert N.device_status() == 0
