"""The request server's threads under ThreadSanitizer on the CPU (no GPU).

final184_gb300/csrc/serve.cpp is compiled unchanged with -fsanitize=thread against tests/cpp/serve_fake_device.cpp
(a host stand-in for the CUDA runtime and the f184gi calls the server makes: streams as queues with completion
times, device memory as host memory) and driven by tests/cpp/serve_tsan_main.cpp: concurrent submitters,
cancellation, statistics polling, host-buffer requests, injected update failures (F184GI_REQ_INJECT_FAIL: that
request fails, its batch runs) and a scheduler thread lost between admission and issue
(F184GI_REQ_INJECT_WORKER_EXIT: queued requests fail with F184GI_ERR_WORKER, later submissions are refused).  Any
data race ThreadSanitizer sees fails the test.  The per-request JSON log (f184gi_server_set_log) is checked too.
"""
import json
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_server_threads_race_free_and_faults_reported(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    exe = str(tmp_path / "serve_tsan")
    src = [os.path.join(ROOT, "final184_gb300", "csrc", "serve.cpp"),
           os.path.join(ROOT, "tests", "cpp", "serve_fake_device.cpp"),
           os.path.join(ROOT, "tests", "cpp", "serve_tsan_main.cpp")]
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-g", "-fsanitize=thread", "-pthread", "-I", cuda_inc,
                        "-I", os.path.join(ROOT, "include"), *src, "-o", exe, "-ldl"], capture_output=True, text=True)
    if r.returncode != 0 and "tsan" in (r.stderr or "").lower():
        pytest.skip("ThreadSanitizer runtime unavailable: " + r.stderr.splitlines()[-1])
    assert r.returncode == 0, r.stderr
    log = str(tmp_path / "requests.jsonl")
    env = dict(os.environ, TSAN_OPTIONS="halt_on_error=1 exitcode=66 second_deadlock_stack=1")
    p = subprocess.run([exe, log], capture_output=True, text=True, env=env, timeout=300)
    assert "ThreadSanitizer" not in p.stderr, p.stderr[-4000:]
    assert p.returncode == 0, (p.returncode, p.stdout, p.stderr[-4000:])
    assert "worker loss reported" in p.stdout
    lines = [json.loads(x) for x in open(log)]
    assert len(lines) >= 100
    assert {"ticket", "scene", "status", "batch", "views", "moves", "pixels", "queued_ms", "latency_ms"} <= set(lines[0])
    assert any(x["status"] == -2 for x in lines) and any(x["status"] == 0 for x in lines)
    assert any(x["status"] == -9 for x in lines)  # the request whose batch the lost worker had admitted
