"""The register-resident top-k list of the tensor-core search (reg_insert in
csrc/search_tc.cu), restated step for step in Python integers: masked-select
shift of the keys, the nibble permutation of dot slots, and the returned k-th
key, checked against a plain sorted list for every k in 1..16."""
import random

M64 = (1 << 64) - 1


def reg_insert(keys, slots, k, key, dot, dots, kr=16):
    pos = sum(1 for i in range(kr - 1) if i < k - 1 and keys[i] > key)
    for i in range(kr - 1, -1, -1):
        prev = keys[i - 1] if i > 0 else 0
        sh = M64 if (pos < i < k) else 0
        at = M64 if i == pos else 0
        keys[i] = (keys[i] & ~(sh | at) & M64) | (prev & sh) | (key & at)
    freed = (slots >> (4 * (k - 1))) & 15
    below = (1 << (4 * pos)) - 1
    thru = M64 if pos >= 15 else (1 << (4 * pos + 4)) - 1
    upto = M64 if k >= 16 else (1 << (4 * k)) - 1
    slots = ((slots & below) | (freed << (4 * pos)) | ((slots << 4) & upto & ~thru & M64)
             | (slots & ~upto & M64)) & M64
    dots[freed] = dot
    last = 0
    for i in range(kr):
        last |= keys[i] & (M64 if i == k - 1 else 0)
    return last, slots


def test_register_list_matches_sorted_list():
    rnd = random.Random(7)
    for trial in range(4000):
        k = 1 + trial % 16
        keys, slots, dots, kth = [0] * 16, 0xfedcba9876543210, [None] * 16, 0
        ref = []
        for j in range(rnd.randint(0, 80)):
            key = rnd.getrandbits(rnd.choice((3, 8, 40))) + 1   # small ranges force near-ties
            if any(key == x for x, _ in ref) or key <= kth:
                continue    # keys are distinct; the kernel inserts only above the k-th
            ref.append((key, j))
            ref.sort(reverse=True)
            ref = ref[:k]
            kth, slots = reg_insert(keys, slots, k, key, j, dots)
        want = ref + [(0, 0)] * (k - len(ref))
        got = [(keys[i], dots[(slots >> (4 * i)) & 15] if keys[i] else 0) for i in range(k)]
        assert got == want, (trial, k)
        assert kth == want[k - 1][0]
        # the first k slot nibbles stay a permutation of 0..k-1
        assert sorted((slots >> (4 * i)) & 15 for i in range(k)) == list(range(k))
