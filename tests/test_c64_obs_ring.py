"""Index logic of the complex64 kernels' observables ring (propagate_c64_smem_kernel and
propagate_c64_kernel in mma_gb300/csrc/tdse_c64.cu), replayed on the CPU: at step k > 0 warp 0
writes output k's float-pair totals to slot (k - 1) mod KB and, when that slot is KB - 1, converts
outputs k - KB + 1 .. k; after the last step it writes output S and converts the (S - 1) mod KB + 1
outputs still pending.  Every output 1..S must be converted exactly once, from the slot that
holds it, for any step count S and block size KB (the number of warps: 8, 16 or 32)."""
import pytest


def replay(S, KB):
    ring = {}
    done = []
    for k in range(S):
        if k > 0:
            ring[(k - 1) % KB] = k  # obs_reduce(k)
            if (k - 1) % KB == KB - 1:  # obs_flush(k, KB)
                done += [(ko, ring[(ko - 1) % KB]) for ko in range(k - KB + 1, k + 1)]
    if S > 0:
        ring[(S - 1) % KB] = S  # obs_reduce(S)
        cnt = (S - 1) % KB + 1  # obs_flush(S, cnt)
        done += [(ko, ring[(ko - 1) % KB]) for ko in range(S - cnt + 1, S + 1)]
    return done


@pytest.mark.parametrize("KB", [8, 16, 32])
def test_every_output_converted_once_from_its_slot(KB):
    for S in list(range(0, 3 * KB + 2)) + [4412, 4413, 8826]:
        done = replay(S, KB)
        assert [ko for ko, _ in done] == list(range(1, S + 1)), S
        assert all(ko == held for ko, held in done), S  # the slot still held that output
