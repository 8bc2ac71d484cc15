"""Generates asg_knn_net.cuh: the comparator networks of k_knn_t33's queue flush.

k_knn_t33 keeps each query's 33 smallest squared distances sorted in
registers.  Candidates below the current 33rd go to a per-lane queue of
KQ = 16 values in shared memory; when one lane's queue is full the warp
merges every lane's queue at once:

  knn_sort16     Batcher's odd-even merge sort of the 16 queued values
                 (63 comparators);
  knn_merge33    Batcher's odd-even merge of the sorted 33 with the sorted
                 16 for arbitrary lengths (Knuth, TAOCP 5.3.4), pruned to the
                 comparators that reach the 34 smallest outputs: the new
                 sorted 33 and the 34th smallest (the smallest value dropped,
                 which tells whether a dropped value ties the new 33rd).

Both networks are checked here by the 0-1 principle (every 0-1 input for the
sort, every pair of sorted 0-1 inputs for the merge) before the header is
written.  Run:  python gen_knn_net.py  (writes asg_knn_net.cuh beside it).
"""
import os

KQ = 16
KA = 33


def oddeven_merge_pow2(lo, n, r, out):
    """Batcher's merge of the sorted halves of wires lo..lo+n-1 (n a power of 2)."""
    step = r * 2
    if step < n:
        oddeven_merge_pow2(lo, n, step, out)
        oddeven_merge_pow2(lo + r, n, step, out)
        for i in range(lo + r, lo + n - r, step):
            out.append((i, i + r))
    else:
        out.append((lo, lo + r))


def oddeven_sort(lo, n, out):
    if n > 1:
        m = n // 2
        oddeven_sort(lo, m, out)
        oddeven_sort(lo + m, m, out)
        oddeven_merge_pow2(lo, n, 1, out)


def merge_any(a, b, out):
    """Batcher's odd-even merge of sorted wire lists a and b of any lengths:
    merge the even-indexed and the odd-indexed subsequences, then one layer of
    comparators (d_i, c_{i+1}).  Returns the wires in merged order."""
    if not a:
        return list(b)
    if not b:
        return list(a)
    if len(a) == 1 and len(b) == 1:
        out.append((a[0], b[0]))
        return [a[0], b[0]]
    c = merge_any(a[0::2], b[0::2], out)
    d = merge_any(a[1::2], b[1::2], out)
    res = [c[0]]
    for i in range(len(d)):
        if i + 1 < len(c):
            out.append((d[i], c[i + 1]))
            res += [d[i], c[i + 1]]
        else:
            res.append(d[i])
    res += c[len(d) + 1:]
    return res


def prune(net, outputs):
    """Keep the comparators that reach the given output wires."""
    need = set(outputs)
    kept = []
    for i, j in reversed(net):
        if i in need or j in need:
            kept.append((i, j))
            need.update((i, j))
    return kept[::-1]


def run(net, x, order=None):
    x = list(x)
    for i, j in net:
        if x[i] > x[j]:
            x[i], x[j] = x[j], x[i]
    return [x[w] for w in order] if order is not None else x


def check_sort(net, n):
    for bits in range(1 << n):
        y = run(net, [(bits >> k) & 1 for k in range(n)])
        if any(y[k] > y[k + 1] for k in range(n - 1)):
            return False
    return True


def check_merge(net, na, nb, order, keep):
    for za in range(na + 1):
        for zb in range(nb + 1):
            x = [0] * za + [1] * (na - za) + [0] * zb + [1] * (nb - zb)
            if run(net, x, order)[:keep] != sorted(x)[:keep]:
                return False
    return True


def networks():
    sort = []
    oddeven_sort(0, KQ, sort)
    assert check_sort(sort, KQ)
    full = []
    order = merge_any(list(range(KA)), list(range(KA, KA + KQ)), full)
    merge = prune(full, order[:KA + 1])
    assert check_merge(merge, KA, KQ, order, KA + 1)
    return sort, merge, order


def header():
    sort, merge, order = networks()
    L = ["// asg_knn_net.cuh -- generated by gen_knn_net.py; do not edit.",
         "// Comparator networks of k_knn_t33's queue flush (checked by the 0-1",
         "// principle in the generator).  A comparator leaves min in x, max in y.",
         "#pragma once",
         "",
         "namespace asg {",
         "",
         f"constexpr int KNN_QUEUE = {KQ};",
         "",
         "#define ASG_CX(x, y) { const float lo_ = fminf(x, y); y = fmaxf(x, y); x = lo_; }",
         "",
         f"// Batcher's odd-even merge sort of v[0..{KQ - 1}] ascending ({len(sort)} comparators)",
         f"__device__ __forceinline__ void knn_sort{KQ}(float (&v)[{KQ}])",
         "{"]
    L += [f"    ASG_CX(v[{i}], v[{j}])" for i, j in sort]
    L += ["}",
          "",
          f"// a[0..{KA - 1}] and v[0..{KQ - 1}] ascending -> a = the {KA} smallest of both,",
          f"// ascending; returns the {KA + 1}th smallest.  Batcher's odd-even merge for",
          f"// lengths {KA} and {KQ}, pruned to the first {KA + 1} outputs ({len(merge)} comparators).",
          f"__device__ __forceinline__ float knn_merge{KA}(float (&a)[{KA}], const float (&v)[{KQ}])",
          "{"]
    L.append("    float " + ", ".join(f"w{i} = a[{i}]" for i in range(KA)) + ";")
    L.append("    float " + ", ".join(f"w{KA + i} = v[{i}]" for i in range(KQ)) + ";")
    L += [f"    ASG_CX(w{i}, w{j})" for i, j in merge]
    L += [f"    a[{p}] = w{order[p]};" for p in range(KA)]
    L += [f"    return w{order[KA]};", "}", "", "#undef ASG_CX", "", "}  // namespace asg", ""]
    return "\n".join(L)


if __name__ == "__main__":
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "asg_knn_net.cuh")
    with open(path, "w") as f:
        f.write(header())
    print("wrote", path)
