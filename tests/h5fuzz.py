"""Test helper: damaged copies of an HDF5 file walked through every reader
entry point of the engine library in a child process (so that a crash or a
hang fails the test instead of ending the test run)."""
import subprocess
import sys

SCRIPT = r'''
import ctypes as C, random, sys
L = C.CDLL(sys.argv[1])
base = open(sys.argv[2], "rb").read()
rng = random.Random(int(sys.argv[3]))
tmp = sys.argv[4]
names = C.create_string_buffer(1 << 16)
def walk(group, depth):
    if depth > 6 or L.wlg_h5_list(tmp.encode(), group.encode(), names, len(names)) != 0:
        return
    for n in names.value.decode(errors="replace").splitlines()[:20]:
        full = group + "/" + n
        if n.endswith("/"):
            walk(full[:-1], depth + 1)
            continue
        t, cnt = C.c_int(0), C.c_ulonglong(0)
        if L.wlg_h5_read(tmp.encode(), full.encode(), C.byref(t), C.byref(cnt), None, C.c_ulonglong(0)) == 0 \
                and cnt.value < (1 << 16):
            out = C.create_string_buffer(cnt.value * 16 + 16)
            L.wlg_h5_read(tmp.encode(), full.encode(), C.byref(t), C.byref(cnt), out, C.c_ulonglong(len(out)))
        a = C.create_string_buffer(4096)
        L.wlg_h5_attribute(tmp.encode(), full.encode(), b"CodeVersion", a, len(a))
for i in range(int(sys.argv[5])):
    b = bytearray(base)
    r = rng.random()
    if r < 0.6:
        for _ in range(rng.randint(1, 4)):
            b[rng.randrange(len(b))] = rng.randrange(256)
    elif r < 0.75:
        b = b[:rng.randrange(len(b))]
    else:
        p = rng.randrange(len(b) - 8)
        b[p:p + 8] = rng.choice([b"\xff" * 8, b"\x00" * 8, rng.randrange(1 << 64).to_bytes(8, "little"),
                                 rng.randrange(len(base)).to_bytes(8, "little")])
    open(tmp, "wb").write(bytes(b))
    walk("", 0)
print("ok")
'''


def check(lib_path, src, tmp_path, seeds=(1, 2), n=300):
    for seed in seeds:
        r = subprocess.run([sys.executable, "-c", SCRIPT, lib_path, str(src), str(seed), str(tmp_path / f"m{seed}.h5"),
                            str(n)], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr[-2000:]
