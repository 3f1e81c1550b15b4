"""numpy model of the device DFT (mma_gb300/csrc/dft.cu), index for index.

Test infrastructure: it restates the kernels' plan (length choice, radix order, Bluestein
tables) and their arithmetic (Stockham passes, real packing and unpacking) so that the index
arithmetic can be checked against numpy.fft on the CPU before it runs on a GPU.

Conventions (FFTW's, which the reference uses through tools_fftw3.c):
    r2c:  X_k = sum_j x_j exp(-2 pi i j k / n),  k = 0 .. n/2
    c2r:  x_j = sum_{k=0}^{n-1} X_k exp(+2 pi i j k / n)  with X_{n-k} = conj(X_k)
"""
import numpy as np

SMOOTH = (2, 3, 5, 7)


def is_smooth(n):
    for p in SMOOTH:
        while n % p == 0:
            n //= p
    return n == 1


def next_smooth(n):
    while not is_smooth(n):
        n += 1
    return n


def radices(M):
    """Radix order of the passes: 8s, then a 4 or a 2 for the rest of the power of two, then 7s,
    5s and 3s (largest first)."""
    out = []
    m = M
    while m % 8 == 0:
        out.append(8)
        m //= 8
    if m % 4 == 0:
        out.append(4)
        m //= 4
    if m % 2 == 0:
        out.append(2)
        m //= 2
    for p in (7, 5, 3):
        while m % p == 0:
            out.append(p)
            m //= p
    assert m == 1, M
    return out


def plan(L):
    """Complex DFT of length L: direct when L is 7-smooth, else Bluestein over the smallest
    7-smooth M >= 2L - 1."""
    if is_smooth(L):
        return dict(L=L, M=L, bluestein=False)
    M = next_smooth(2 * L - 1)
    return dict(L=L, M=M, bluestein=True)


def twiddles(M):
    j = np.arange(M)
    return np.exp(-2j * np.pi * j / M)  # device: sincospi(-2 j / M)


def stockham(x, tw, rads):
    """Forward DFT of x (length M) by Stockham autosort passes, as the kernels run them:
    pass with radix R, Ns = product of the earlier radices; butterfly j < M/R reads
    x[j + r M/R], multiplies value r by w^(r k) (w = exp(-2 pi i / (Ns R)), k = j mod Ns),
    applies DFT_R and writes value r to (j // Ns) Ns R + k + r Ns."""
    M = len(x)
    a = x.astype(np.complex128).copy()
    Ns = 1
    for R in rads:
        b = np.empty_like(a)
        MR = M // R
        step = M // (Ns * R)  # table stride of w
        for j in range(MR):
            k = j % Ns
            v = np.array([a[j + r * MR] * tw[(r * k * step) % M] for r in range(R)])
            # DFT_R with roots exp(-2 pi i m / R) = tw[m M / R]
            y = np.array([sum(v[r] * tw[((r * q) % R) * (M // R)] for r in range(R)) for q in range(R)])
            base = (j // Ns) * Ns * R + k
            for r in range(R):
                b[base + r * Ns] = y[r]
        a = b
        Ns *= R
    return a


def stockham_vec(x, tw, rads):
    """The same passes vectorised over the butterflies (identical index arithmetic)."""
    M = len(x)
    a = x.astype(np.complex128).copy()
    Ns = 1
    for R in rads:
        MR = M // R
        j = np.arange(MR)
        k = j % Ns
        step = M // (Ns * R)
        v = np.stack([a[j + r * MR] * tw[(r * k * step) % M] for r in range(R)])
        roots = np.array([[tw[((r * q) % R) * (M // R)] for r in range(R)] for q in range(R)])
        y = roots @ v
        base = (j // Ns) * Ns * R + k
        b = np.empty_like(a)
        for r in range(R):
            b[base + r * Ns] = y[r]
        a = b
        Ns *= R
    return a


def bluestein_tables(L, M):
    j = np.arange(L)
    c = np.exp(-1j * np.pi * ((j * j) % (2 * L)) / L)  # device: sincospi(-(j^2 mod 2L) / L)
    b = np.zeros(M, dtype=np.complex128)
    b[:L] = np.conj(c)
    b[M - L + 1:] = np.conj(c[1:])[::-1]
    B = stockham_vec(b, twiddles(M), radices(M)) / M
    return c, B


def cdft(z, p):
    """Forward complex DFT of length L by the plan."""
    L, M = p["L"], p["M"]
    tw = twiddles(M)
    rads = radices(M)
    if not p["bluestein"]:
        return stockham_vec(z, tw, rads)
    c, B = bluestein_tables(L, M)
    a = np.zeros(M, dtype=np.complex128)
    a[:L] = z * c
    A = stockham_vec(a, tw, rads) * B
    conv = np.conj(stockham_vec(np.conj(A), tw, rads))  # inverse by conjugation (1/M is in B)
    return conv[:L] * c


def rfft(x):
    """r2c of a real row of length n (FFTW convention), n/2 + 1 outputs."""
    n = len(x)
    if n % 2:
        Z = cdft(x.astype(np.complex128), plan(n))
        return Z[:n // 2 + 1]
    L = n // 2
    z = x[0::2] + 1j * x[1::2]
    Z = cdft(z, plan(L))
    k = np.arange(L + 1)
    Zk = Z[k % L]
    Zc = np.conj(Z[(L - k) % L])
    w = np.exp(-2j * np.pi * k / n)  # device: sincospi(-2 k / n)
    return 0.5 * (Zk + Zc) - 0.5j * w * (Zk - Zc)


def irfft(X, n):
    """c2r of length n from X[0 .. n/2] (FFTW convention: unnormalised, Hermitian extension)."""
    if n % 2:
        full = np.zeros(n, dtype=np.complex128)
        h = n // 2 + 1
        full[:h] = X[:h]
        full[h:] = np.conj(X[1:n - h + 1][::-1])
        full[0] = X[0].real
        y = np.conj(cdft(np.conj(full), plan(n)))
        return y.real
    L = n // 2
    k = np.arange(L)
    Xk = X[k].copy()
    Xk[0] = X[0].real  # FFTW ignores the imaginary parts of the DC and Nyquist bins
    Xn = np.conj(X[L - k])
    Xn[0] = X[L].real
    w = np.exp(2j * np.pi * k / n)
    Z = (Xk + Xn) + 1j * w * (Xk - Xn)
    z = np.conj(cdft(np.conj(Z), plan(L)))
    out = np.empty(n)
    out[0::2] = z.real
    out[1::2] = z.imag
    return out
