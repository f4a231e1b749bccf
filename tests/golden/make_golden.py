"""Writes tests/golden/kat.json: known-answer cases taken from portBLAS's own
tests and documentation, with the expected outputs derived analytically
(exact integer arithmetic) — independent of both the oracle and the CUDA
kernels, so either can be pinned against them.

Sources (paths in the portBLAS source tree):
  * iamax/iamin generation modes Limit / Incrementing / Decrementing at the
    sizes and increments of test/unittest/blas1/blas1_iaminmax_common.hpp:31-87;
    iamax fills Limit with 0.0 (test/unittest/blas1/blas1_iamax_test.cpp:17),
    iamin with numeric_limits<T>::max() (blas1_iamin_test.cpp:40-44); incx < 0
    returns 0 (src/interface/blas1_interface.hpp:375-378).
  * the 3x3 AddOperator example of doc/Reduction.md:26-50, plus the other five
    operators on the same matrix (src/operations/blas_operators.hpp:149-274).
  * GEMM alpha == 0 / beta == 0 rules (src/interface/gemm_interface.hpp:112-139,
    src/operations/blas3/gemm_local.hpp:401-409) on small integer matrices
    whose products are exact in FP32.
  * asum / dot / nrm2 on integer vectors with exact answers, including the
    negative-increment view rule of src/views/view.hpp:43-48.

Run: python tests/golden/make_golden.py  (deterministic; no inputs needed)
"""
import json
import math
import os

FLT_MAX = 3.4028234663852886e38


def iaminmax_cases():
    cases = []
    for size in (11, 65, 1000000):
        for inc in (1, -1, 5):
            for mode in ("limit", "incrementing", "decrementing"):
                for op in ("iamax", "iamin"):
                    if inc < 0:
                        exp = 0
                    elif mode == "limit":
                        exp = 0  # all |x| equal: first index
                    elif mode == "incrementing":  # buffer[i] = i, logical x_j = buffer[j*inc]
                        exp = size - 1 if op == "iamax" else 0
                    else:  # buffer[i] = len-1-i
                        exp = 0 if op == "iamax" else size - 1
                    fill = 0.0 if op == "iamax" else FLT_MAX
                    cases.append(dict(op=op, n=size, incx=inc, mode=mode, fill=fill, expected=exp))
    return cases


def reduction_cases():
    # doc/Reduction.md: column-major data 1..9 shown as the matrix
    #   1 4 7 / 2 5 8 / 3 6 9
    data = [float(v) for v in range(1, 10)]
    rows = cols = 3
    col = [[data[i + 3 * j] for i in range(3)] for j in range(3)]
    row = [[data[i + 3 * j] for j in range(3)] for i in range(3)]
    f = {
        "add": lambda v: sum(v),
        "product": lambda v: math.prod(v),
        "max": max,
        "min": min,
        "abs_add": lambda v: sum(abs(x) for x in v),
        "mean": lambda v: sum(v) / len(v),
    }
    cases = []
    for op, fn in f.items():
        cases.append(dict(op=op, dim="inner", rows=rows, cols=cols, ld=3, data=data, expected=[fn(c) for c in col]))
        cases.append(dict(op=op, dim="outer", rows=rows, cols=cols, ld=3, data=data, expected=[fn(r) for r in row]))
    # ld > rows (ld = 2*rows, padding entries must be ignored)
    padded = []
    for j in range(3):
        padded += col[j] + [1e30, -1e30, 7.0]
    cases.append(dict(op="add", dim="inner", rows=3, cols=3, ld=6, data=padded, expected=[6.0, 15.0, 24.0]))
    cases.append(dict(op="add", dim="outer", rows=3, cols=3, ld=6, data=padded, expected=[12.0, 15.0, 18.0]))
    return cases


def gemm_cases():
    # A (3x2), B (2x4), C (3x4), column-major, small integers
    M, N, K = 3, 4, 2
    A = [1.0, -2.0, 3.0, 4.0, 0.0, -1.0]              # A(i,k) = A[i + 3k]
    B = [2.0, 1.0, -3.0, 5.0, 0.0, 2.0, 1.0, -1.0]    # B(k,j) = B[k + 2j]
    Cin = [float(v) for v in range(1, 13)]
    AB = [[sum(A[i + 3 * k] * B[k + 2 * j] for k in range(K)) for j in range(N)] for i in range(M)]

    def out(alpha, beta, c):
        r = []
        for j in range(N):
            for i in range(M):
                if alpha == 0.0:
                    r.append(0.0 if beta == 0.0 else beta * c[i + 3 * j])
                else:
                    r.append(alpha * AB[i][j] + (0.0 if beta == 0.0 else beta * c[i + 3 * j]))
        return r

    cases = []
    for alpha, beta in ((1.0, 0.0), (1.5, 0.5), (0.0, 2.0), (0.0, 0.0), (2.0, 1.0)):
        cases.append(dict(ta="n", tb="n", m=M, n=N, k=K, alpha=alpha, beta=beta, a=A, lda=3, b=B, ldb=2, c=Cin,
                          ldc=3, c_nan=False, expected=out(alpha, beta, Cin)))
    # beta == 0 must not read C (NaN in C must not leak); alpha == 0, beta == 0 writes zeros
    for alpha in (1.0, 0.0):
        cases.append(dict(ta="n", tb="n", m=M, n=N, k=K, alpha=alpha, beta=0.0, a=A, lda=3, b=B, ldb=2, c=Cin,
                          ldc=3, c_nan=True, expected=out(alpha, 0.0, Cin)))
    # transposed operands: A^T stored as K x M (lda 2), B^T stored as N x K (ldb 4)
    At = [A[i + 3 * k] for i in range(M) for k in range(K)]   # At[k + 2i] = A(i,k)
    Bt = [B[k + 2 * j] for k in range(K) for j in range(N)]   # Bt[j + 4k] = B(k,j)
    cases.append(dict(ta="t", tb="t", m=M, n=N, k=K, alpha=1.0, beta=1.0, a=At, lda=2, b=Bt, ldb=4, c=Cin, ldc=3,
                      c_nan=False, expected=out(1.0, 1.0, Cin)))
    cases.append(dict(ta="T", tb="c", m=M, n=N, k=K, alpha=1.0, beta=0.0, a=At, lda=2, b=Bt, ldb=4, c=Cin, ldc=3,
                      c_nan=False, expected=out(1.0, 0.0, Cin)))
    return cases


def blas1_cases():
    x = [3.0, -4.0, 12.0, 0.0, -84.0]       # |x|: 3 4 12 0 84 ; sqrt(9+16+144+7056) = 85
    y = [1.0, 2.0, -1.0, 5.0, 0.5]
    cases = [
        dict(op="asum", n=5, incx=1, x=x, expected=103.0),
        dict(op="nrm2", n=5, incx=1, x=x, expected=85.0),
        dict(op="dot", n=5, incx=1, incy=1, x=x, y=y, expected=3.0 - 8.0 - 12.0 + 0.0 - 42.0),
        # stride 2 over [3, _, 12, _, -84]; negative stride reverses the view
        dict(op="asum", n=3, incx=2, x=x, expected=99.0),
        dict(op="asum", n=3, incx=-2, x=x, expected=99.0),
        dict(op="dot", n=3, incx=2, incy=-2, x=x, y=y,
             expected=3.0 * 0.5 + 12.0 * -1.0 + -84.0 * 1.0),  # y view reversed: y[4], y[2], y[0]
        dict(op="nrm2", n=2, incx=1, x=[3e30, 4e30], expected=5e30),      # overflow-safe scaling
        dict(op="nrm2", n=2, incx=1, x=[3e-30, 4e-30], expected=5e-30),   # underflow-safe scaling
        dict(op="iamax", n=5, incx=1, x=[1.0, -7.0, 7.0, 2.0, -7.0], expected=1),  # ties -> first
        dict(op="iamin", n=5, incx=1, x=[5.0, -1.0, 3.0, 1.0, -1.0], expected=1),
    ]
    return cases


def main():
    out = dict(iaminmax=iaminmax_cases(), reduction=reduction_cases(), gemm=gemm_cases(), blas1=blas1_cases())
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kat.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(path, {k: len(v) for k, v in out.items()})


if __name__ == "__main__":
    main()
