"""CPU models of the launch schedules of the group kernels (no GPU).

* k_fz_shared (fft_method_test_gb300/csrc/fft_fast.cuh): a CTA walks items
  (tile, member), member fastest.  Before transforming item i its thread 0
  issues the TMA copies of item i + 1: the spectral boxes into stage
  (i + 1) & 1 and, when i + 1 starts a tile, the Green tile into Green buffer
  ((i + 1) // G) & 1.  The model replays that order and checks that no copy
  lands in a buffer an unfinished item still reads, and that every item reads
  the Green tile of its own tile.
* group launches: the grid dimensions and the member index each kernel takes
  from blockIdx stay inside the member tables the host writes.
"""
import pytest


def _replay_shared_z(G, tiles):
    """Events of one CTA with `tiles` tiles and G members; returns the
    (item -> green tile read) map and raises on a hazard."""
    n = tiles * G
    stage_owner = {}   # stage -> item whose data it holds
    green_owner = {}   # green buffer -> tile whose Green it holds
    done = set()
    read_green = {}

    def issue(i):
        st = i & 1
        prev = stage_owner.get(st)
        assert prev is None or prev in done, ("stage overwritten", i, prev)
        stage_owner[st] = i
        if i % G == 0:
            gb = (i // G) & 1
            prev_t = green_owner.get(gb)
            if prev_t is not None:
                # every item of the previous tile in this buffer has finished
                assert all(j in done for j in range(prev_t * G, prev_t * G + G)), ("green overwritten", i)
            green_owner[gb] = i // G

    if n:
        issue(0)
    for i in range(n):
        if i + 1 < n:
            issue(i + 1)
        # transform item i: its stage and its tile's Green buffer
        assert stage_owner[i & 1] == i
        read_green[i] = green_owner[(i // G) & 1]
        done.add(i)
    return read_green


@pytest.mark.parametrize("G", [1, 2, 3, 5, 16])
@pytest.mark.parametrize("tiles", [0, 1, 2, 3, 7])
def test_shared_green_z_pass_schedule_has_no_buffer_hazard(G, tiles):
    reads = _replay_shared_z(G, tiles)
    assert len(reads) == G * tiles
    for i, t in reads.items():
        assert t == i // G  # the Green tile of the item's own tile


@pytest.mark.parametrize("members", [1, 2, 3, 16])
def test_group_member_indices_stay_in_the_tables(members):
    # y pass: grid.z = 3 * members, member = blockIdx.z // 3, comp = blockIdx.z % 3
    zs = range(3 * members)
    assert {z // 3 for z in zs} == set(range(members))
    assert {z % 3 for z in zs} == {0, 1, 2}
    # tensor maps: [2 m] spectral, [2 m + 1] Green, 2 * members entries
    assert max(2 * m + 1 for m in range(members)) < 2 * members
    # vector kernels: grid (max_blocks, members); blocks past a member's own
    # count return before touching its buffers
    nblk = [7, 3, 12][: members] + [5] * max(0, members - 3)
    max_blocks = max(nblk)
    for m in range(members):
        active = [b for b in range(max_blocks) if b < nblk[m]]
        assert len(active) == nblk[m]
