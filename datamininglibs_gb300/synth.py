"""Seeded synthetic stand-ins for the benchmark workloads.

Every generator returns ``X`` as float32 in the reference's feature-major layout
``[n_features, n_rows]`` (``samples[f*N + i]``, lib_parsing/source/csv_parser.cc:92-96)
and ``y`` as float32 (a class index stored as a float, as in ``MlDataFrame<float>``,
or a regression target).  ``n_rows`` can be lowered to make small parity cases of
the same distributions.
"""
import numpy as np


def ert_binary(n_rows=4601, n_features=57, seed=0):
    """Zero-inflated lognormal features, ~39% positive labels.

    Each value is 0 with p=0.7, else lognormal(mu=-1, sigma=1.5); the label is
    1 when a seeded random linear combination of log1p(x) exceeds its 61st
    percentile, then flipped with p=0.05."""
    rng = np.random.default_rng(seed)
    zero = rng.random((n_features, n_rows)) < 0.7
    vals = rng.lognormal(mean=-1.0, sigma=1.5, size=(n_features, n_rows))
    X = np.where(zero, 0.0, vals).astype(np.float32)
    w = rng.standard_normal(n_features)
    score = w @ np.log1p(X.astype(np.float64))
    thr = np.percentile(score, 61.0)
    y = (score > thr).astype(np.int32)
    flip = rng.random(n_rows) < 0.05
    y = np.where(flip, 1 - y, y)
    return X, y.astype(np.float32)


def rf_multiclass(n_rows=1_000_000, n_features=128, n_classes=10, n_int=16, seed=0):
    """N(0,1) features with ``n_int`` of them replaced by integers 0..15 stored as
    float; labels = argmax(x @ W + Gumbel noise) with a seeded W."""
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n_features, n_rows), dtype=np.float32)
    cols = rng.choice(n_features, size=min(n_int, n_features), replace=False)
    for c in cols:
        X[c] = rng.integers(0, 16, size=n_rows).astype(np.float32)
    W = rng.standard_normal((n_features, n_classes)).astype(np.float32)
    logits = X.T @ W
    logits += rng.gumbel(size=(n_rows, n_classes)).astype(np.float32)
    y = np.argmax(logits, axis=1).astype(np.float32)
    return X, y


def rf_regression(n_rows=4_000_000, n_features=64, seed=0):
    """U(0,1) features; y = sum_{k=1..8} sin(2*pi*x_k*k) + 0.5*x_9*x_10 + N(0, 0.1^2)."""
    rng = np.random.default_rng(seed)
    X = rng.random((n_features, n_rows), dtype=np.float32)
    y = np.zeros(n_rows, np.float64)
    col = lambda j: X[j % n_features].astype(np.float64)  # noqa: E731 (fewer than 10 features)
    for k in range(1, 9):
        y += np.sin(2.0 * np.pi * col(k - 1) * k)
    y += 0.5 * col(8) * col(9)
    y += rng.normal(0.0, 0.1, size=n_rows)
    return X, y.astype(np.float32)


def uneven_problems(n_problems=256, seed=0, n_range=(200, 50_000), f_range=(8, 256),
                    c_range=(2, 8)):
    """Independent classification problems of uneven sizes: rows log-uniform in
    ``n_range``, features uniform in ``f_range``, classes uniform in ``c_range``;
    N(0,1) features, labels = argmax of a seeded random linear map."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_problems):
        n = int(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1]))))
        f = int(rng.integers(f_range[0], f_range[1] + 1))
        c = int(rng.integers(c_range[0], c_range[1] + 1))
        X = rng.standard_normal((f, n), dtype=np.float32)
        W = rng.standard_normal((f, c)).astype(np.float32)
        y = np.argmax(X.T @ W, axis=1).astype(np.float32)
        out.append((X, y, c))
    return out


def request_rows(rng, n_rows, n_features, kind):
    """Feature-major rows for a prediction request, drawn like the training data."""
    if kind == "ert_binary":
        zero = rng.random((n_features, n_rows)) < 0.7
        vals = rng.lognormal(mean=-1.0, sigma=1.5, size=(n_features, n_rows))
        return np.where(zero, 0.0, vals).astype(np.float32)
    if kind == "rf_regression":
        return rng.random((n_features, n_rows), dtype=np.float32)
    return rng.standard_normal((n_features, n_rows), dtype=np.float32)
