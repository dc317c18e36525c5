"""The flush's key order in two 32-bit sort words (stc_lsm.cu, sort_keys /
low_word / high_word), emulated in numpy without a GPU: a stable sort by the
low word, then by the high word, must give the order of the reference's key
(over, sid, pid, target, duration, end) -- CTF keys by sid:12 | pid:26 |
target:26 | duration:32 | end:32 (cuda/geometry.cu:724-726, 799-806), then
the oversize keys by theirs with sid 0."""
import numpy as np
import pytest


def bits_for(x):
    return max(int(x), 1).bit_length()


def words(pid, target, dur, end, over, rank, N, max_end, max_dur):
    eb, db, ib = bits_for(max_end), bits_for(max_dur), bits_for(N - 1 if N > 1 else 1)
    assert eb + db < 32
    low_t = 32 - eb - db
    th = ib - low_t if ib > low_t else 0
    assert 1 + ib + th <= 32
    m32 = np.uint64(0xFFFFFFFF)
    u = lambda a: a.astype(np.uint64)
    low = (u(end) | (u(dur) << np.uint64(eb)) | (u(target) << np.uint64(eb + db))) & m32
    major = np.where(over, pid, rank[pid]).astype(np.uint64)
    high = (np.where(over, np.uint64(1) << np.uint64(ib + th), np.uint64(0)) | (major << np.uint64(th)) |
            ((u(target) >> np.uint64(low_t)) if th else np.uint64(0))) & m32
    return low.astype(np.uint32), high.astype(np.uint32)


# two-word cases only (eb + db < 32 and 1 + ib + th <= 32; wider keys take the
# per-field words): no high target bits; 3M and 10M objects at step-sized end
# times; the 32-bit limit of the high word exactly; two objects
@pytest.mark.parametrize("N,max_end,max_dur", [(1000, 200, 50), (3_000_000, 300, 60), (10_000_000, 100, 60),
                                               (10_000_000, 1023, 31), (2, 3, 1)])
def test_two_word_order_is_the_key_order(N, max_end, max_dur):
    rng = np.random.default_rng(N)
    K = 200_000
    # few objects and times so that many keys tie on the leading fields
    objs = rng.integers(0, N, min(N, 3000))
    pid = rng.choice(objs, K)
    target = rng.choice(objs, K)
    end = rng.integers(0, max_end + 1, K)
    dur = rng.integers(0, max_dur + 1, K)
    over = rng.random(K) < 0.05
    sid = rng.integers(1, 101, N)  # per object
    # the objects' rank in (sid, pid) order
    order = np.lexsort((np.arange(N), sid))
    rank = np.empty(N, np.int64)
    rank[order] = np.arange(N)
    low, high = words(pid, target, dur, end, over, rank, N, max_end, max_dur)
    by_words = np.lexsort((np.arange(K), low, high))
    sid_eff = np.where(over, 0, sid[pid])
    by_key = np.lexsort((np.arange(K), end, dur, target, pid, sid_eff, over))
    assert np.array_equal(by_words, by_key)
