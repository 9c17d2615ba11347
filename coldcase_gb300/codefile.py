"""Code-file format of the reference (one codeword per line).

Base-36 digits, MSB first, one character per coordinate; or integers
separated by spaces, commas or tabs for q > 36.  '#' starts a comment.
  * read_code   -- covsearch2e's reader (cov/engine/covsearch2e.c:870-898):
                   characters that are not base-36 digits are skipped, a
                   line's length must be n;
  * parse_code  -- verify_cov's reader (cov/verify_cov.py:60-92): strict,
                   de-duplicated, returns (codewords, n_duplicates);
  * distinct_code / write_code -- covsearch2e's writer (:791-853): exactly M
                   distinct words (duplicates dropped in order, topped up with
                   the lowest unused word indices), written to <path>.part and
                   renamed into place.
"""
import os
import re

import numpy as np

_LEADING_INT = re.compile(r"[+-]?\d+")

DIGITS = "0123456789abcdefghijklmnopqrstuvwxyz"
_DIGVAL = {c: i for i, c in enumerate(DIGITS)}


class CodeFileError(ValueError):
    pass


def count_code(path):
    """Lines holding at least one base-36 digit (covsearch2e.c:900-914)."""
    m = 0
    with open(path) as f:
        for line in f:
            line = line.split("#")[0]
            if any(ch in _DIGVAL for ch in line):
                m += 1
    return m


def read_code(path, n):
    """covsearch2e --in reader; returns uint8 array (m, n)."""
    rows = []
    with open(path) as f:
        for line in f:
            line = line.split("#")[0]
            if any(ch in line for ch in " ,\t"):
                toks = [t for t in line.replace(",", " ").replace("\t", " ").split() if t]
                # atoi: the leading integer of the token (0 if none), then
                # the uint8_t cast of the reader (modulo 256)
                w = []
                for t in toks[:n]:
                    m = _LEADING_INT.match(t)
                    w.append((int(m.group(0)) if m else 0) & 0xff)
            else:
                w = [_DIGVAL[ch] for ch in line.rstrip("\r\n") if ch in _DIGVAL][:n]
            if not w:
                continue
            if len(w) != n:
                raise CodeFileError("%s: bad codeword length %d" % (path, len(w)))
            rows.append(w)
    if not rows:
        return np.zeros((0, n), dtype=np.uint8)
    return np.array(rows, dtype=np.uint8)


def parse_code(path, q, n):
    """verify_cov reader: (list of tuples, number of duplicate lines)."""
    words = []
    with open(path) as f:
        for lineno, raw in enumerate(f, 1):
            line = raw.split("#")[0].strip()
            if not line:
                continue
            if any(ch in line for ch in " ,\t"):
                try:
                    w = [int(t) for t in line.replace(",", " ").split() if t]
                except ValueError:
                    raise CodeFileError("%s:%d: cannot parse %r" % (path, lineno, line))
            else:
                w = []
                for ch in line:
                    k = DIGITS.find(ch.lower())
                    if k < 0:
                        raise CodeFileError("%s:%d: bad digit %r" % (path, lineno, ch))
                    w.append(k)
            if len(w) != n:
                raise CodeFileError("%s:%d: length %d, expected n=%d" % (path, lineno, len(w), n))
            for v in w:
                if not 0 <= v < q:
                    raise CodeFileError("%s:%d: digit %d out of range for q=%d" % (path, lineno, v, q))
            words.append(tuple(w))
    if not words:
        raise CodeFileError("%s: no codewords" % path)
    uniq = list(dict.fromkeys(words))
    return uniq, len(words) - len(uniq)


def read_code_finisher(path, q, n, M):
    """covcount's reader (cov/engine/covcount.c:94-118): at most M words;
    lines of the wrong length or with a digit >= q are skipped, not errors;
    a missing file reads as no words."""
    rows = []
    try:
        f = open(path)
    except OSError:
        return np.zeros((0, n), dtype=np.uint8)
    with f:
        for line in f:
            if len(rows) >= M:
                break
            line = line.split("#")[0]
            if any(ch in line for ch in " ,\t"):
                toks = [t for t in line.replace(",", " ").replace("\t", " ").split() if t][:n]
                w = []
                for t in toks:
                    m = _LEADING_INT.match(t)
                    w.append((int(m.group(0)) if m else 0) & 0xff)
            else:
                w = [_DIGVAL[ch] for ch in line.rstrip("\r\n") if ch in _DIGVAL][:n]
            if len(w) != n or any(v >= q for v in w):
                continue
            rows.append(w)
    if not rows:
        return np.zeros((0, n), dtype=np.uint8)
    return np.array(rows, dtype=np.uint8)


def word_index(code, q):
    code = np.asarray(code, dtype=np.int64)
    n = code.shape[1]
    w = q ** np.arange(n - 1, -1, -1, dtype=np.int64)
    return code @ w


def distinct_code(code, q, n, M):
    """Exactly M distinct words: duplicates dropped in order, topped up with
    the lowest unused word indices (covsearch2e.c:799-837)."""
    code = np.asarray(code, dtype=np.uint8).reshape(-1, n)[:M]
    idx = word_index(code, q) if len(code) else np.zeros(0, dtype=np.int64)
    seen = set()
    keep = []
    for k, x in enumerate(idx.tolist()):
        if x in seen:
            continue
        seen.add(x)
        keep.append(k)
    out = [code[k] for k in keep]
    N = q ** n
    x = 0
    pw = [q ** (n - 1 - j) for j in range(n)]
    while len(out) < M and x < N:
        if x not in seen:
            seen.add(x)
            out.append(np.array([(x // pw[j]) % q for j in range(n)], dtype=np.uint8))
        x += 1
    if not out:
        return np.zeros((0, n), dtype=np.uint8)
    return np.stack(out).astype(np.uint8)


def format_code(code, q):
    lines = []
    for row in np.asarray(code):
        if q <= 36:
            lines.append("".join(DIGITS[int(v)] for v in row))
        else:
            lines.append(" ".join(str(int(v)) for v in row))
    return "".join(s + "\n" for s in lines)


def write_code(path, code, q, n, M):
    """Atomic publication of M distinct words (write .part, rename)."""
    body = format_code(distinct_code(code, q, n, M), q)
    tmp = path + ".part"
    with open(tmp, "w") as f:
        f.write(body)
        f.flush()
    os.replace(tmp, path)
