"""The autotuner's coordinate descent without a GPU: a stand-in handle whose
per-pass and per-step times are known functions of the launch shape."""
from rocflupicl_gb300 import autotune as AT
from rocflupicl_gb300 import engine as E


class FakeHandle:
    """set_tuning / profile / timer calls of a region handle; each step of the
    current shape adds known times to the per-kernel profile and the timer."""

    def __init__(self, pass_ms, step_ms):
        self.pass_ms, self.step_ms = pass_ms, step_ms
        self.shape = {k: 0 for k in E.TUNING_KEYS}
        self.prof_on, self.prof, self.timer, self.steps, self.applied = False, {}, 0.0, 0, []

    def set_tuning(self, **kw):
        assert set(kw) <= set(E.TUNING_KEYS)
        self.shape = dict(self.shape, **kw)
        self.applied.append(dict(self.shape))

    def step(self):
        self.steps += 1
        self.timer += self.step_ms(self.shape)
        if self.prof_on:
            for k, f in self.pass_ms.items():
                t, n = self.prof.get(k, (0.0, 0))
                self.prof[k] = (t + 3 * f(self.shape), n + 3)   # three stages per step

    def sync(self):
        pass

    def profile(self, on=True):
        self.prof_on = on
        if on:
            self.prof = {}

    def profile_read(self):
        return dict(self.prof)

    def timer_start(self):
        self.timer = 0.0

    def timer_stop(self):
        return self.timer


def _fake():
    pref = {"gradBlock": 64, "faceBlock": 128, "cellBlock": 256}
    pass_ms = {
        "gradient": lambda s: 1.7 + 0.01 * abs((s["gradBlock"] or 128) - pref["gradBlock"]) / 64,
        "face_flux": lambda s: 0.63 + 0.02 * abs((s["faceBlock"] or 128) - pref["faceBlock"]) / 64
        + 0.01 * ((s["facesPerThread"] or 1) - 1),
        "gather_update": lambda s: 0.58 + 0.01 * abs((s["cellBlock"] or 128) - pref["cellBlock"]) / 64,
    }

    def step_ms(s):
        base = 8.8 + (0.5 if s["gridCap"] else 0.0)
        return base + (0.9 if s["persistentStage"] else 0.0)
    return FakeHandle(pass_ms, step_ms), pref


def test_descent_picks_each_knobs_fastest_candidate():
    h, pref = _fake()
    knobs = {"gradBlock": AT.BLOCKS, "faceBlock": AT.BLOCKS, "facesPerThread": (1, 2),
             "cellBlock": AT.BLOCKS, "gridCap": (0, 608, 1216)}
    out = AT._descend(h, h.step, 3, knobs, persistent=True)
    shape = out["shape"]
    assert shape["gradBlock"] == pref["gradBlock"] and shape["faceBlock"] == pref["faceBlock"]
    assert shape["cellBlock"] == pref["cellBlock"] and shape["facesPerThread"] == 1
    assert shape["gridCap"] == 0 and shape["persistentStage"] == 0
    # every candidate was timed, per pass for the block knobs, per step for the grid
    assert set(out["ms"]["gradBlock"]) == set(AT.BLOCKS)
    assert abs(out["ms"]["gridCap"][608] - 9.3) < 1e-12
    assert out["ms"]["persistentStage"][1] > out["ms"]["persistentStage"][0]
    # steps: (steps + 1 settle step) per candidate, two whole-step trials at the end
    n_cands = sum(len(v) for v in knobs.values())
    assert out["steps_taken"] == n_cands * 4 + 2 * 4 == h.steps
    assert h.shape == shape                       # the kept shape is the one left applied


def test_persistent_stage_kept_when_faster():
    h, _ = _fake()
    h.step_ms = lambda s: 9.0 - (0.5 if s["persistentStage"] else 0.0)
    out = AT._descend(h, h.step, 2, {"gridCap": (0, 608)}, persistent=True)
    assert out["shape"]["persistentStage"] == 1
    # the cooperative shape keeps the default blocks and the grid cap chosen before it
    assert all(out["shape"][k] == 0 for k in ("gradBlock", "faceBlock", "cellBlock"))
