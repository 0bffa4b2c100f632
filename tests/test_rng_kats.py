"""Known answers of the random generators under KMeans::kmeans_plus_plus
(src/rand_custom.rs:8-32 with rand 0.8.5, which the reference tree does not
vendor), checked primitive by primitive against the published algorithms'
own test outputs, so that the draws no longer rest only on two restatements
agreeing with each other:

  - SplitMix64 (Steele, Lea & Flood), the filler of SmallRng::seed_from_u64;
  - xoshiro256++ (Blackman & Vigna), SmallRng on 64-bit targets: the output
    sequence of the authors' reference implementation from state {1, 2, 3, 4};
  - the ChaCha quarter round and block function (RFC 7539 sections 2.1.1 and
    2.3.2, 20 rounds); StdRng runs the same block function with 12 rounds;
  - PCG32's XSH-RR output (O'Neill), whose step fills StdRng's key in
    seed_from_u64: the pcg32 demo's first outputs for srandom(42, 54).

The library's own restatement (csrc/host_rng.cpp) is tied to these through
test_capi_cpu.py, which requires its draws and raw streams to equal the
oracle's for both generators and many seeds.
"""
import numpy as np

import oracle


def test_splitmix64_from_zero():
    assert [int(v) for v in oracle.splitmix64(0, 3)] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4,
                                                        0x06C45D188009454F]


def test_xoshiro256pp_reference_outputs():
    # The first two follow by hand from the definition: rotl(1 + 4, 23) + 1 =
    # 41943041; after one update s = {7, 0, 262146, 6 << 45}, so
    # rotl(7 + (6 << 45), 23) + 7 = (7 << 23) + 96 + 7 = 58720359.
    want = [41943041, 58720359, 3588806011781223, 3591011842654386, 9228616714210784205,
            9973669472204895162, 14011001112246962877, 12406186145184390807, 15849039046786891736,
            10450023813501588000]
    assert [int(v) for v in oracle.xoshiro256pp([1, 2, 3, 4], 10)] == want


def test_chacha_quarter_round_rfc7539():
    got = oracle.chacha_quarter_round(0x11111111, 0x01020304, 0x9B8D6F43, 0x01234567)
    assert got == [0xEA2A92F4, 0xCB1CF8CE, 0x4581472E, 0x5881C4BB]


def test_chacha20_block_rfc7539():
    key = np.frombuffer(bytes(range(32)), dtype="<u4")
    nonce = np.frombuffer(bytes([0, 0, 0, 9, 0, 0, 0, 0x4A, 0, 0, 0, 0]), dtype="<u4")
    out = oracle.chacha_block(key, [1, nonce[0], nonce[1], nonce[2]], 20)
    want = bytes.fromhex(
        "10f1e7e4d13b5915500fdd1fa32071c4c7d1f4c733c068030422aa9ac3d46c4e"
        "d2826446079faa0914c2d705d98b02a2b5129cd1de164eb9cbd083e8a2503c4e")
    assert out.astype("<u4").tobytes() == want


def test_chacha12_is_the_same_block_function():
    # StdRng's block: 12 rounds, 64-bit counter in words 12-13, stream 0.  Its
    # first words for seed 0 come from the same function the 20-round vector pins.
    key = np.zeros(8, np.uint32)
    k = oracle.pcg32(0, 11634580456548205067, 8, after_step=True)
    block = oracle.chacha_block(k, [0, 0, 0, 0], 12)
    raw = oracle.rng_u64(2, seed=0, rng=oracle.RNG_STD)
    assert int(raw[0]) == (int(block[1]) << 32) | int(block[0])
    assert int(raw[1]) == (int(block[3]) << 32) | int(block[2])
    assert not np.array_equal(oracle.chacha_block(key, [0, 0, 0, 0], 12), oracle.chacha_block(key, [0, 0, 0, 0], 20))


def test_pcg32_demo_outputs():
    # pcg32_srandom(42, 54): inc = 54 * 2 + 1, state = 0, step, state += 42, step
    inc, mul, mask = 109, 6364136223846793005, (1 << 64) - 1
    st = (0 * mul + inc) & mask
    st = (st + 42) & mask
    st = (st * mul + inc) & mask
    want = [0xA15C02B7, 0x7B47F409, 0xBA1D3330, 0x83D2F293, 0xBFA4784B, 0xCBED606E]
    assert [int(v) for v in oracle.pcg32(st, inc, 6)] == want


def test_small_rng_draws_from_the_pinned_primitives():
    # SmallRng::seed_from_u64(s): state = four SplitMix64 outputs; next_u64 = xoshiro256++
    for seed in (0, 42, 2**63 + 5):
        state = oracle.splitmix64(seed, 4)
        assert np.array_equal(oracle.rng_u64(16, seed=seed, rng=oracle.RNG_SMALL), oracle.xoshiro256pp(state, 16))
