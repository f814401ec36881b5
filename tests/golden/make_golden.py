"""Regenerate known_answers.json from the reference's own sources.

The reference ships three known answers for this path, all as text in its
sources (read here as text; nothing of the reference is executed):
  * accelerate-llvm-ptx/test/nofib/Data/Array/Accelerate/LLVM/PTX/NoFib/RunQ.hs:
    `A.sum (A.map (+1) xs)` over xs = [1..n], n = 10000, must equal
    n * (n + 1) `div` 2 + n (= 50015000);
  * accelerate-llvm-native/src/Data/Array/Accelerate/LLVM/Native/CodeGen/Scan.hs:
    the example `scanl (+) 10 (use $ fromList (Z :. 10) [0..])`
    ==> Array (Z :. 11) [10,10,11,13,16,20,25,31,38,46,55];
  * the same file (and PTX/CodeGen/Scan.hs): the example of mkScan',
    "Variant of 'scanl' where the final result is returned in a separate
    array", ==> ( Array (Z :. 10) [10,10,11,13,16,20,25,31,38,46], Array Z [55] ).
    Its expression is spelled `scanr' (+) 10 ...`, but the text and the values
    are those of scanl' (exclusive from the left, total 55 apart), so it is
    recorded as a scanl' known answer.
Run:  python tests/golden/make_golden.py path/to/accelerate-llvm-checkout
"""
import json
import pathlib
import re
import sys

if len(sys.argv) != 2:
    sys.exit("usage: make_golden.py path/to/accelerate-llvm-checkout")
ref = pathlib.Path(sys.argv[1])
runq = (ref / "accelerate-llvm-ptx/test/nofib/Data/Array/Accelerate/LLVM/PTX/NoFib/RunQ.hs").read_text()
scan = (ref / "accelerate-llvm-native/src/Data/Array/Accelerate/LLVM/Native/CodeGen/Scan.hs").read_text()

assert "A.sum (A.map (+1)" in runq
n = int(re.search(r"let n = (\d+)", runq).group(1))
assert "n * (n + 1) `div` 2 + n" in runq
total = n * (n + 1) // 2 + n

m2 = re.search(r"scanl \(\+\) (\d+) \(use \$ fromList \(Z :\. (\d+)\) \[0\.\.\]\)\s*\n-- >\s*\n-- > ==> Array \(Z :\. (\d+)\) \[([0-9,]+)\]", scan)
seed, cnt, n_out, vals = int(m2.group(1)), int(m2.group(2)), int(m2.group(3)), [int(v) for v in m2.group(4).split(",")]

m3 = re.search(r"-- Variant of 'scanl' where the final result is returned in a separate array\.\s*\n--\s*\n"
               r"-- > scanr' \(\+\) (\d+) \(use \$ fromList \(Z :\. (\d+)\) \[0\.\.\]\)\s*\n-- >\s*\n"
               r"-- > ==> \( Array \(Z :\. (\d+)\) \[([0-9,]+)\]\s*\n--\s*, Array Z \[(\d+)\]", scan)
seed3, cnt3, n_out3 = int(m3.group(1)), int(m3.group(2)), int(m3.group(3))
vals3, total3 = [int(v) for v in m3.group(4).split(",")], int(m3.group(5))

golden = {
    "sum_map_succ": {"source": "accelerate-llvm-ptx/test/nofib/Data/Array/Accelerate/LLVM/PTX/NoFib/RunQ.hs",
                     "input_range": [1, n], "map": "+1", "op": "+", "seed": 0, "expect": total},
    "scanl_example": {"source": "accelerate-llvm-native/src/Data/Array/Accelerate/LLVM/Native/CodeGen/Scan.hs",
                      "op": "+", "seed": seed, "input": list(range(cnt)), "expect": vals, "out_len": n_out},
    "scanl_prime_example": {"source": "accelerate-llvm-native/src/Data/Array/Accelerate/LLVM/Native/CodeGen/Scan.hs",
                            "note": "spelled scanr' in the source; text and values are scanl'",
                            "op": "+", "seed": seed3, "input": list(range(cnt3)), "expect": vals3,
                            "expect_total": total3, "out_len": n_out3},
}
out = pathlib.Path(__file__).with_name("known_answers.json")
out.write_text(json.dumps(golden) + "\n")
print(out, total, vals, vals3, total3)
