"""Rewrites the kernel launches of a CUDA source for the host launch emulation
(tests/host_build/cuda_emu.h), test infrastructure only:

    kernel<T, U><<<grid, block, smem, stream>>>(args)
 -> ::cuda_emu::launch(grid, block, kernel<T, U>)(args)

Everything else of the source is left as it is."""

from __future__ import annotations


def _split_top_level(s: str) -> list[str]:
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch in "(<[":
            depth += 1
        elif ch in ")>]":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur.strip())
            cur = ""
        else:
            cur += ch
    parts.append(cur.strip())
    return parts


def emulate_launches(src: str) -> str:
    out, i = [], 0
    while True:
        j = src.find("<<<", i)
        if j < 0:
            out.append(src[i:])
            return "".join(out)
        # the kernel expression before the launch: a name with template arguments
        k, depth = j, 0
        while k > 0:
            ch = src[k - 1]
            if ch == ">":
                depth += 1
            elif ch == "<":
                depth -= 1
            elif depth == 0 and not (ch.isalnum() or ch in "_:"):
                break
            k -= 1
        kernel = src[k:j]
        e = src.find(">>>", j)
        cfg = _split_top_level(src[j + 3:e])
        out.append(src[i:k])
        out.append(f"::cuda_emu::launch({cfg[0]}, {cfg[1]}, {kernel})")
        i = e + 3


def rewrite(source_path: str, target_path: str) -> None:
    with open(source_path) as f:
        src = f.read()
    with open(target_path, "w") as f:
        f.write(emulate_launches(src))
