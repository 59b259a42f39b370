"""Host-side logic that needs no GPU: the autotuner's choice rule, the kernel-variant flags of the Python
binding, and the argument checks of the entry points added for the work-queue forward and the fused
gradient-Adam (they return their status before any CUDA call), and that the package never reaches into the
oracle."""
import ctypes
import os

import pytest

from bats_gb300 import kernels as K
from bats_gb300.autotune import _choose

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BAD_SHAPE, NULLPTR, WORKSPACE = 1, 2, 4


def test_autotuner_ties_go_to_the_first_candidate():
    order = ["tile", "lanes", "queue"]
    assert _choose({"tile": 1.00, "lanes": 2.0, "queue": 0.99}, order) == "tile"      # within 3 %
    assert _choose({"tile": 1.00, "lanes": 2.0, "queue": 0.90}, order) == "queue"     # clearly faster
    assert _choose({"tile": 0.005, "lanes": 0.05, "queue": 0.004}, order) == "tile"   # within 2 us
    assert _choose({"tile": 0.010, "lanes": 0.05, "queue": 0.004}, order) == "queue"


def test_forward_variant_flags():
    assert K.is_queue_algo(K.FWD_QUEUE) and K.is_queue_algo(K.FWD_QUEUE64)
    assert K.is_queue_algo(K.FWD_QUEUE | K.FWD_NO_PAD | K.FWD_STAGE)
    assert not K.is_queue_algo(K.FWD_TILE | K.FWD_STAGE) and not K.is_queue_algo(K.FWD_LANES)
    assert K.FWD_STAGE & K.FWD_NO_PAD == 0 and K.FWD_STAGE & 0xff == 0


@pytest.fixture(scope="module")
def lib():
    from bats_gb300 import _lib
    try:
        return _lib.load()
    except RuntimeError as exc:  # pragma: no cover - the library is built by build()
        pytest.skip(str(exc))


def _fwd_queue(L, batch=4, n_post=8, ld=8, algo=0, ws=16, ws_bytes=1 << 20):
    fake = ctypes.c_void_p(256)  # never dereferenced: the checks below return first
    return L.bats_lif_forward_fc_queue(fake, fake, 64, fake, ld, batch, n_post, 4, 1.0, 1.0, 0.26, 0.2, fake, fake,
                                       fake, fake, fake, algo, ctypes.c_void_p(ws) if ws else None, ws_bytes, None)


def test_work_queue_forward_argument_checks(lib):
    L = lib
    assert L.bats_lif_forward_fc_queue_workspace_bytes(0) == 256
    assert L.bats_lif_forward_fc_queue_workspace_bytes(4096) == 256 + 4096 * 4
    assert L.bats_lif_forward_fc_queue_workspace_bytes(33) == 256 + 256
    assert _fwd_queue(L, batch=0) == 0                      # nothing to do
    assert _fwd_queue(L, ld=6) == BAD_SHAPE                 # ld not a multiple of 4
    assert _fwd_queue(L, algo=K.FWD_LANES) == BAD_SHAPE     # the queue runs the tile kernels only
    assert _fwd_queue(L, ws=0) == NULLPTR
    assert _fwd_queue(L, ws=8) == WORKSPACE                 # not 16-byte aligned
    assert _fwd_queue(L, ws_bytes=64) == WORKSPACE          # below bats_lif_forward_fc_queue_workspace_bytes
    assert b"workspace" in L.bats_last_error()


def _grad_adam(L, group=8, ld=128, n_post=100, batch=32, ws_bytes=0, grad=True, heads=None):
    fake = ctypes.c_void_p(256)
    return L.bats_weights_gradient_adam(fake, fake, None, None, 1000, fake, fake, fake, heads, batch, n_post, 4, 50, group,
                                        fake if grad else None, fake, fake, 0.9, 0.999, 1e-8, 1e-3, fake, fake, fake,
                                        ld, fake if ws_bytes else None, ws_bytes, None)


def test_fused_gradient_adam_argument_checks(lib):
    L = lib
    assert _grad_adam(L, group=1) == BAD_SHAPE              # the batch mean needs groups of >= 2 samples
    assert _grad_adam(L, ld=64) == BAD_SHAPE                # the transposed copy's rows hold n_post
    assert _grad_adam(L, batch=0) == 0
    assert _grad_adam(L) == WORKSPACE                       # 4 partials need the workspace
    assert _grad_adam(L, group=64, grad=False) == NULLPTR   # one partial lives in grad
    assert _grad_adam(L, heads=ctypes.c_void_p(264)) == BAD_SHAPE  # cursor heads not 16-byte aligned


def _step_stand_in(batch, sizes, groups, algos):
    """An FCTrainStep's launch list and variant choices without its device buffers."""
    import types
    from bats_gb300.train import FCLayerSpec, FCTrainStep
    ts = FCTrainStep.__new__(FCTrainStep)
    ts.B = batch
    ts.specs = [FCLayerSpec(n, 0.13, 1.0, 1.0, 30) for n in sizes[1:]]
    ts.ev = [types.SimpleNamespace(n_neurons=n) for n in sizes[:-1]]
    ts.groups = list(groups)
    ts.fwd_algo = list(algos)
    L = len(sizes) - 1
    names = ["adam.powers"]
    for i in range(1, L + 1):  # batches wider than the sort's resident CTAs: the hidden layers' sample order
        names += ([f"L{i}.order"] if i > 1 and batch > 2 * 152 else []) + [f"L{i}.sort", f"L{i}.forward"]
    names += ["loss"]
    for i in range(L, 0, -1):
        names += [f"L{i}.prep"] + ([f"L{i}.pre_err"] if i > 1 else []) + [f"L{i}.grad_adam"]
    ts.launches = [(n, None) for n in names]
    return ts


def test_launch_count_matches_the_launch_lists():
    """gpu_launches of the bench: the kernels of one train step, as ncu lists them (profiles/
    train_step_launches_*.md): 21 for the literal 784-800-800-10 step, 16 for the 1024-1024-20 uneven batch
    with the output layer on the work queue (the second layer's sort takes its samples longest first)."""
    lit = _step_stand_in(256, (784, 800, 800, 10), (32, 32, 16), (K.FWD_TILE | K.FWD_STAGE, K.FWD_TILE, K.FWD_TILE))
    assert lit.launches_per_step == 21
    bat = _step_stand_in(4096, (1024, 1024, 20), (64, 16), (K.FWD_TILE, K.FWD_QUEUE))
    assert bat.launches_per_step == 16


def test_product_does_not_import_the_oracle():
    """The oracle is test infrastructure: no module of the package imports it, and no native source includes
    anything from it."""
    import ast
    pkg = os.path.join(ROOT, "bats_gb300")
    offenders = []
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            path = os.path.join(dirpath, f)
            if f.endswith(".py"):
                tree = ast.parse(open(path).read(), filename=path)
                for node in ast.walk(tree):
                    names = ([a.name for a in node.names] if isinstance(node, ast.Import)
                             else [node.module or ""] if isinstance(node, ast.ImportFrom) else [])
                    if any(n == "oracle" or n.startswith("oracle.") for n in names):
                        offenders.append(path)
            elif f.endswith((".cu", ".cuh", ".h", ".cpp")):
                if any(line.lstrip().startswith("#include") and "oracle" in line for line in open(path)):
                    offenders.append(path)
    assert not offenders, offenders


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """Without the built library every entry point raises: there is no fallback to compute elsewhere."""
    from bats_gb300 import _lib
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "libbats_gb300.so"))
    with pytest.raises(RuntimeError, match="missing"):
        _lib.load()
    with pytest.raises(RuntimeError, match="missing"):
        _lib.call("bats_abi_version")


def test_caller_outputs_are_checked_before_any_call():
    """An `out` tensor that the kernels could not fill in row-major order is refused with ValueError before
    the library is called (here: host tensors, a wrong shape, a transposed view)."""
    from types import SimpleNamespace
    import torch
    post = torch.zeros((2, 3, 4))
    ev = SimpleNamespace(n_neurons=5, k=1, cap=5)
    with pytest.raises(ValueError, match="contiguous CUDA"):
        K.weights_gradient(ev, post, None, 5, per_sample=True, out=torch.zeros((2, 3, 5)))
    with pytest.raises(ValueError, match="contiguous CUDA"):
        K.weights_gradient(ev, post, None, 5, per_sample=False, group=2, out=torch.zeros((5, 3)).t())
    with pytest.raises(ValueError, match="contiguous CUDA"):
        K.pre_errors(ev, None, post, None, 0.13, 0.26, out=torch.zeros((2, 5, 2)))
    assert K._out.__doc__


def test_two_stream_enqueue_order(monkeypatch):
    """enqueue_launches: the side launches run on the second stream, each after an event recorded on the
    main stream right after its dependency; the main stream waits for the second before the first staged
    weights copy; everything else keeps the list's order on the main stream; without a second stream the
    list runs in order on the main one."""
    import torch
    from bats_gb300 import train

    log = []

    class FakeEvent:
        def __init__(self, *a, **k):
            self.after = None

        def record(self, stream):
            self.after = list(log)
            log.append(("record", stream.name))

    class FakeStream:
        def __init__(self, name, handle):
            self.name, self.cuda_stream = name, handle

        def wait_event(self, e):
            log.append(("wait_event", self.name, e.after[-1]))

        def wait_stream(self, other):
            log.append(("wait_stream", self.name, other.name))

    monkeypatch.setattr(torch.cuda, "Event", FakeEvent)
    names = ["L3.prep", "L3.pre_err", "L3.grad_adam", "L2.prep", "L2.pre_err", "L2.grad_adam", "L1.prep",
             "L1.grad_adam", "L3.wt_copy", "L2.wt_copy"]
    launches = [(n, (lambda s, n=n: log.append((n, s)))) for n in names]
    side = {"L3.grad_adam": "L3.prep", "L2.grad_adam": "L2.prep"}
    main, aux = FakeStream("main", 1), FakeStream("aux", 2)
    train.enqueue_launches(launches, side, main, aux)
    assert log == [("L3.prep", 1), ("record", "main"), ("L3.pre_err", 1),
                   ("wait_event", "aux", ("L3.prep", 1)), ("L3.grad_adam", 2),
                   ("L2.prep", 1), ("record", "main"), ("L2.pre_err", 1),
                   ("wait_event", "aux", ("L2.prep", 1)), ("L2.grad_adam", 2),
                   ("L1.prep", 1), ("L1.grad_adam", 1), ("wait_stream", "main", "aux"),
                   ("L3.wt_copy", 1), ("L2.wt_copy", 1)]
    log.clear()
    train.enqueue_launches(launches, side, main, None)
    assert log == [(n, 1) for n in names]
