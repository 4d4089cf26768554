"""Interpreter exit with a context whose stream another library wraps: a torch
pinned tensor copied on an ExternalStream of the context's stream, alive at
exit. The library's exit handler must leave the stream alone (torch releases
such tensors after it), so the process exits cleanly."""
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

SCRIPT = """
import sys
sys.path.insert(0, %r)
import torch
import futspace_gb300 as fs
ctx = fs.Context(0)
stream = torch.cuda.ExternalStream(ctx.stream_handle, device=0)
dev = torch.empty(1 << 20, dtype=torch.int32, device='cuda')
host = torch.empty(1 << 20, dtype=torch.int32, pin_memory=True)
hm = fs.gen_heights(3, 64, 0.55)
fmap = fs.Map(ctx, hm, fs.gen_colors(4, hm, 12))
with torch.cuda.stream(stream):
    host.copy_(dev, non_blocking=True)
frame = ctx.render(fmap, fs.gen_cameras(5, hm, 1, screen_h=24)[0], 32, 24)
torch.cuda.synchronize()
print("ok", int(frame.sum() > 0))
"""


def test_exit_with_wrapped_stream_alive():
    pytest.importorskip("torch")
    r = subprocess.run([sys.executable, "-c", SCRIPT % str(ROOT)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip().startswith("ok")
