"""pz_explicit_terms_noalloc, the entry point for callers that cannot
allocate device memory (a host capturing its own CUDA graph, or one whose
device memory all belongs to its own pool allocator).

It must give the same explicit terms as pz_explicit_terms, which takes its
intermediates from cudaMallocAsync, on consecutive calls (the static scratch
array keeps the previous call's contents), and it must refuse instances
larger than its fixed array.  This file is collected last so that a run which
stops at the first failure has run every other test before it.
"""
import numpy as np
import pytest

from tests.helpers import gpu_config, oracle, rel_err, seeded

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.fixture(scope="module")
def pz():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pizza_gb300 import build as b
    b.build()
    import pizza_gb300
    return pizza_gb300


def _state(spec, seed, steps):
    sim = oracle(spec, temp0=seeded(spec, seed))
    for _ in range(steps):
        sim.advance()
    return {f: getattr(sim, f).copy() for f in ("us", "up", "om", "temp")}


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls(pz):
    import torch
    specs = [dict(n_r_max=33, m_max=32, ek=1e-3, ra=1e5, l_ek_pump=True, dtMax=1e-4, matrix_solve="INFLUENCE"),
             dict(n_r_max=65, m_max=96, ek=1e-4, ra=2e6, l_ek_pump=True, dtMax=2e-5, matrix_solve="INFLUENCE")]
    ens = pz.Ensemble([gpu_config(s) for s in specs])
    # two different states per instance, so the second call overwrites what the first left behind
    for call in range(2):
        for i, s in enumerate(specs):
            st = _state(s, seed=20 + 10 * call + i, steps=2 + call)
            dev = {f: torch.from_numpy(np.ascontiguousarray(st[f].T)).cuda() for f in st}
            torch.cuda.synchronize()
            ref = ens.explicit_terms(i, dev["us"], dev["up"], dev["om"], dev["temp"])
            got = ens.explicit_terms(i, dev["us"], dev["up"], dev["om"], dev["temp"], noalloc=True)
            ens.sync()
            for k in range(4):
                a, b = got[k].cpu().numpy(), ref[k].cpu().numpy()
                assert rel_err(a, b) <= TOL, f"call {call} instance {i} output {k}"


def test_noalloc_rejects_instances_beyond_its_array(pz):
    import torch
    spec = dict(n_r_max=128, m_max=256, ek=1e-3, ra=1e5, dtMax=1e-5, matrix_solve="INFLUENCE")
    ens = pz.Ensemble(gpu_config(spec))
    n, m = 128, 257      # 32896 > PZ_NOALLOC_MAX_MN = 32768
    z = torch.zeros((n, m), dtype=torch.complex128, device="cuda")
    with pytest.raises(pz.PizzaError) as e:
        ens.explicit_terms(0, z, z, z, z, noalloc=True)
    assert e.value.code == -1 and "exceeds the maximum" in str(e.value)
