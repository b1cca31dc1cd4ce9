"""CPU tests of the serving wrapper's bookkeeping, against a stand-in for the
native server (no device): caller tags come back on completion even when
they repeat, a request's buffers stay referenced exactly while it is in
flight, and a refused submission holds nothing."""
import pytest

from althea_gb300 import ibl, serving

torch = pytest.importorskip("torch")


class _FakeNative:
    """The althea_ibl_server_* calls the wrapper makes, held in Python.
    Completions come back in reverse submission order; a request wider than
    `refuse_width` is refused with ERR_BUDGET."""

    def __init__(self, refuse_width=1 << 30):
        self.pending = []  # native tags submitted, not yet completed
        self.refuse_width = refuse_width

    def althea_ibl_server_create(self, cfg_ref, out_ref):
        out_ref._obj.value = 1234
        return ibl.OK

    def althea_ibl_server_submit(self, s, req_ref):
        req = req_ref._obj
        if req.env_width > self.refuse_width:
            return ibl.ERR_BUDGET
        self.pending.append(req.tag)
        return ibl.OK

    def complete(self):
        done, self.pending = list(reversed(self.pending)), []
        self.ready = done

    def althea_ibl_server_poll(self, s, out, cap, n_ref):
        ready = getattr(self, "ready", [])
        k = min(cap, len(ready))
        for i in range(k):
            out[i] = ibl.Completion(ready[i], ibl.OK, 1.0, 2.0, 3.0)
        self.ready = ready[k:]
        n_ref._obj.value = k
        return ibl.OK

    def althea_ibl_server_get_stats(self, s, st_ref):
        st_ref._obj.inflight = len(self.pending)
        st_ref._obj.queued = 0
        return ibl.OK

    def althea_ibl_server_destroy(self, s):
        return ibl.OK

    def althea_ibl_last_error(self):
        return b"refused by the stand-in"


@pytest.fixture
def fake(monkeypatch):
    native = _FakeNative(refuse_width=512)
    native.servers = []
    monkeypatch.setattr(ibl, "load", lambda *a, **k: native)
    yield native
    for server in native.servers:  # closed while the stand-in is still in place
        server.close()

def _server(native):
    server = serving.ProbeServer(budget_bytes=1 << 30)
    native.servers.append(server)
    return server


def _buffers(w):
    h = w // 2
    sizes = serving.mip_sizes_for(w, h, 2)
    mips = torch.zeros(sum(a * b * 4 for a, b in sizes))
    return serving.RequestBuffers(torch.zeros((h, w, 4)), mips, torch.zeros((16, 32, 4)), sizes)


def test_tags_map_back_and_buffers_are_released(fake):
    server = _server(fake)
    bufs = [_buffers(64) for _ in range(3)]
    for tag, b in zip([7, 7, 3], bufs):  # a repeated tag
        server.submit(tag, b)
    assert len(server._inflight) == 3
    assert {id(b) for _, b in server._inflight.values()} == {id(b) for b in bufs}
    assert server.poll() == []
    fake.complete()
    comps = server.poll()
    assert sorted(c.tag for c in comps) == [3, 7, 7]
    assert all(c.status == ibl.OK and c.done_s == 3.0 for c in comps)
    assert server._inflight == {}


def test_refused_submission_holds_nothing(fake):
    server = _server(fake)
    with pytest.raises(ibl.IBLError) as e:
        server.submit(1, _buffers(1024))
    assert e.value.status == ibl.ERR_BUDGET
    assert server._inflight == {}
    server.submit(2, _buffers(64))
    fake.complete()
    assert [c.tag for c in server.poll()] == [2]


def test_poll_returns_more_than_one_batch_of_completions(fake):
    server = _server(fake)
    b = _buffers(32)
    n = 2 * len(server._done) + 5  # more completions than one native poll returns
    for i in range(n):
        server.submit(i, b)
    fake.complete()
    assert sorted(c.tag for c in server.poll()) == list(range(n))
    assert server._inflight == {}
