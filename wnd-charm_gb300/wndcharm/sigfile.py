"""Signature (.sig) and training-set (.fit) text files, byte-compatible with
wndchrm's own writers and readers.

.sig (signatures::SaveToFile / LoadFromFilep, src/wndchrm_src/signatures.cpp:229-307):
    "<class>\\t<version>.<feature vector type>"   (or "<value %f>\\t..." when continuous)
    "<image path>"
    "<value %.8g>\\t<feature name>"               one line per feature (name optional)

.fit (TrainingSet::SaveToFile / ReadFromFile, src/wndchrm_src/TrainingSet.cpp:339-497):
    "<n classes>\\t<version>.<feature vector type>"
    "<n features>"
    "<n samples>"
    feature names, one per line
    class labels 0..n classes, one per line (label 0 is the unknown class, often empty)
    per sample: the values separated by single spaces ("%ld" when the value is
    integral, else "%.8g"), then the class ("%d", or "%f" for a continuous set),
    newline, then the image path on its own line.

Feature vector types: 1 = short (1059 features), 2 = long (2919); version 4.
"""
import math

import numpy as np

FEATURE_VERSION = 4
FV_SHORT, FV_LONG = 1, 2


def _g8(v):
    """C printf("%.8g") of a double (Python's %-formatting follows C for finite values)."""
    v = float(v)
    if math.isnan(v):
        return "nan"
    if math.isinf(v):
        return "inf" if v > 0 else "-inf"
    return "%.8g" % v


def _fit_value(v):
    """A .fit value: "%ld" of the value when it equals its int conversion, else "%.8g"."""
    v = float(v)
    if math.isfinite(v) and abs(v) < 2147483648.0 and v == int(v):
        return "%d" % int(v)
    return _g8(v)


def format_sig(values, names=None, sample_class=0, full_path="", version=FEATURE_VERSION, fv_type=FV_LONG,
               continuous_value=None):
    head = ("%f" % continuous_value) if continuous_value is not None else "%d" % int(sample_class)
    out = ["%s\t%d.%d\n" % (head, version, fv_type), "%s\n" % full_path]
    if names is None:
        out += ["%s\n" % _g8(v) for v in values]
    else:
        if len(names) != len(values):
            raise ValueError("names and values differ in length")
        out += ["%s\t%s\n" % (_g8(v), n) for v, n in zip(values, names)]
    return "".join(out)


def write_sig(path, values, names=None, sample_class=0, full_path="", version=FEATURE_VERSION, fv_type=FV_LONG,
              continuous_value=None):
    with open(path, "w") as f:
        f.write(format_sig(values, names, sample_class, full_path, version, fv_type, continuous_value))


def parse_sig(text, continuous=False):
    """Returns dict(values, names, sample_class, sample_value, version, fv_type, full_path).
    A file without a version on its first line is version 1, type unknown (0)."""
    lines = text.split("\n")
    first = lines[0].split()
    cls, value = 1, None
    if continuous:
        value = float(first[0])
    else:
        cls = int(first[0])
    version, fv_type = 1, 0
    if len(first) > 1 and "." in first[1]:
        maj, mi = first[1].split(".", 1)
        if int(maj) != 0:
            version, fv_type = int(maj), int(mi)
    full_path = lines[1].rstrip("\r") if len(lines) > 1 else ""
    values, names = [], []
    for ln in lines[2:]:
        ln = ln.rstrip("\r")
        if not ln:
            continue
        parts = ln.split("\t", 1) if "\t" in ln else ln.split(None, 1)
        values.append(float(parts[0]))
        names.append(parts[1].strip() if len(parts) > 1 else "")
    return {"values": np.array(values), "names": names, "sample_class": cls, "sample_value": value,
            "version": version, "fv_type": fv_type, "full_path": full_path}


def read_sig(path, continuous=False):
    with open(path) as f:
        return parse_sig(f.read(), continuous)


def format_fit(X, classes, names, class_labels, paths, version=FEATURE_VERSION, fv_type=FV_LONG,
               continuous_values=None):
    """X: samples x features; classes: 1-based class per sample (ignored for a
    continuous set); class_labels: labels 0..n_classes (label 0 first)."""
    X = np.asarray(X, dtype=np.float64)
    n_classes = len(class_labels) - 1
    out = ["%d\t%d.%d\n" % (n_classes, version, fv_type), "%d\n" % X.shape[1], "%d\n" % X.shape[0]]
    out += ["%s\n" % n for n in names]
    out += ["%s\n" % c for c in class_labels]
    for i in range(X.shape[0]):
        row = "".join(_fit_value(v) + " " for v in X[i])
        tail = ("%f" % continuous_values[i]) if continuous_values is not None else "%d" % int(classes[i])
        out.append(row + tail + "\n")
        out.append("%s\n" % paths[i])
    return "".join(out)


def write_fit(path, X, classes, names, class_labels, paths, version=FEATURE_VERSION, fv_type=FV_LONG,
              continuous_values=None):
    with open(path, "w") as f:
        f.write(format_fit(X, classes, names, class_labels, paths, version, fv_type, continuous_values))


def parse_fit(text):
    """Returns dict(X, classes, names, class_labels, paths, version, fv_type)."""
    lines = text.split("\n")
    first = lines[0].split()
    n_classes = int(first[0])
    version, fv_type = 1, 0
    if len(first) > 1 and "." in first[1]:
        maj, mi = first[1].split(".", 1)
        if int(maj) != 0:
            version, fv_type = int(maj), int(mi)
    nf, ns = int(lines[1]), int(lines[2])
    k = 3
    names = [ln.rstrip("\r") for ln in lines[k:k + nf]]
    k += nf
    labels = [ln.rstrip("\r") for ln in lines[k:k + n_classes + 1]]
    k += n_classes + 1
    X = np.zeros((ns, nf))
    classes = np.zeros(ns, dtype=np.int32)
    paths = []
    for i in range(ns):
        tok = lines[k].split()
        X[i] = [float(t) for t in tok[:nf]]
        classes[i] = int(float(tok[nf])) if len(tok) > nf else 0
        paths.append(lines[k + 1].rstrip("\r") if k + 1 < len(lines) else "")
        k += 2
    return {"X": X, "classes": classes, "names": names, "class_labels": labels, "paths": paths,
            "version": version, "fv_type": fv_type}


def read_fit(path):
    with open(path) as f:
        return parse_fit(f.read())
