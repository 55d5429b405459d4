"""Train the learned first correction of the mixed v-Poisson solve on the
config-4 workload and write its weights.

    python -m trans_bl_gb300.learn_config4 [--out DIR] [--crops N] [--iters N]

Config 4: the 1025 x 193 x 32 grid of config 2 at F = 1e-4.  The solver
collects the training data itself while it steps (host-launched steps with
tb_learn_sample): 16 random 72 x 72 crops per solve of the network's input
planes and the exact correction of the warm-start guess, N crops in all
(20000 by default), from a disturbed state past the forcing ramp.  The first
75% of the crops (the earlier steps) train the network with the library's
own kernels (tb_learn_train, Adam); the last 25% are held out.  Then, from a
later state, the run is repeated without the network, with it in every
solve, and gated, and again at F = 1.2e-4 with the same weights, reporting
corrections per step, the share of solves that kept the network's
correction and (gated) the share that ran it.

Writes DIR/learned_config4.f32 (the weight vector, float32) and
DIR/learned_config4.json (the numbers above).
"""
import argparse
import json
import os
import time

import numpy as np

from . import api, configs

HERE = os.path.dirname(os.path.abspath(__file__))


def corrections(ctx, t0, n):
    v0 = ctx.poisson_stats()["total_vcycles"]
    t1 = time.perf_counter()
    for q in range(n):
        ctx.step(t0 + q)
    ctx.synchronize()
    return ctx.poisson_stats()["total_vcycles"] - v0, (time.perf_counter() - t1) / n


def compare(cfg, coefs, base, state, t, w, steps):
    out = {}
    for name, mode in (("without", 0), ("every_solve", 1), ("gated", 2)):
        c = api.Context(cfg, coefs, base)
        if mode:
            c.learn_set_weights(w)
            c.learn_enable(True, gated=(mode == 2))
        c.put_state(state)
        corrections(c, t - 2, 2)                        # warm-start history
        n, sec = corrections(c, t, steps)
        st = c.learn_stats() if mode else {}
        out[name] = {"corrections_per_step": n / steps, "ms_per_step_host": 1e3 * sec}
        if mode:
            out[name].update({"kept": st["kept"], "tried": st["tried"],
                              "kept_share": st["kept"] / max(st["tried"], 1)})
            if mode == 2:
                out[name].update({"evaluated": st["evaluated"], "solves": st["solves"],
                                  "fallback_rate": 1.0 - st["evaluated"] / max(st["solves"], 1)})
        c.close()
    return out


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--out", default=os.path.join(HERE, "data"))
    p.add_argument("--crops", type=int, default=20000)
    p.add_argument("--iters", type=int, default=4000)
    p.add_argument("--eval-steps", type=int, default=16)
    p.add_argument("--weights", default=None,
                   help="evaluate these weights (float32 file) instead of training; writes learned_config4_eval.json")
    a = p.parse_args()
    cfg = configs.config2(tol=1e-10, precision=api.FORM_MIXED)
    coefs, base = configs.setup_inputs(cfg)
    if a.weights:
        w = np.fromfile(a.weights, dtype=np.float32)
        g = api.Context(cfg, coefs, base)
        g.put_state(configs.disturbed_state(cfg, base, np.random.default_rng(41)))
        t = cfg.stpp + 1
        for q in range(8):
            g.step(t + q)
        state = g.get_state()
        g.close()
        res = {"weights": os.path.basename(a.weights), "F_1e-4": compare(cfg, coefs, base, state, t + 10, w, a.eval_steps)}
        cfg2 = configs.config2(tol=1e-10, precision=api.FORM_MIXED, F=1.2e-4)
        coefs2, base2 = configs.setup_inputs(cfg2)
        st2 = configs.disturbed_state(cfg2, base2, np.random.default_rng(42))
        res["F_1.2e-4"] = compare(cfg2, coefs2, base2, st2, cfg2.stpp + 3, w, a.eval_steps)
        os.makedirs(a.out, exist_ok=True)
        json.dump(res, open(os.path.join(a.out, "learned_config4_eval.json"), "w"), indent=1)
        print(json.dumps(res))
        return
    g = api.Context(cfg, coefs, base)
    g.put_state(configs.disturbed_state(cfg, base, np.random.default_rng(41)))
    t = cfg.stpp + 1
    g.learn_init(11)
    per = 16
    g.learn_sample(a.crops, crops_per_solve=per, seed=13)
    steps = 0
    t0 = time.perf_counter()
    while g.learn_stats()["samples"] < a.crops:
        g.step(t + steps)
        steps += 1
    g.learn_sample(0)
    t_sample = time.perf_counter() - t0
    n = g.learn_stats()["samples"]
    ntr = int(0.75 * n)
    g.learn_train(1, batch=32, lr=1e-12, n_train=ntr)      # sets the input and output scales
    l0, guess = g.learn_eval(ntr, n - ntr)
    t0 = time.perf_counter()
    g.learn_train(a.iters, batch=32, lr=1e-3, n_train=ntr)
    t_train = time.perf_counter() - t0
    l1, _ = g.learn_eval(ntr, n - ntr)
    w = g.learn_weights()
    state, t_after = g.get_state(), t + steps
    g.close()
    res = {"workload": "config 4: nx=1025 ny=193 kfour=32, F=1e-4, tol=1e-10, %d steps per period" % cfg.stpp,
           "crops": int(n), "sampling_steps": steps, "train_crops": ntr, "iters": a.iters,
           "sampling_s": t_sample, "training_s": t_train,
           "held_out_defect_vs_guess": {"untrained": l0 / guess, "trained": l1 / guess},
           "F_1e-4": compare(cfg, coefs, base, state, t_after + 2, w, a.eval_steps)}
    cfg2 = configs.config2(tol=1e-10, precision=api.FORM_MIXED, F=1.2e-4)
    coefs2, base2 = configs.setup_inputs(cfg2)
    st2 = configs.disturbed_state(cfg2, base2, np.random.default_rng(42))
    res["F_1.2e-4"] = compare(cfg2, coefs2, base2, st2, cfg2.stpp + 3, w, a.eval_steps)
    os.makedirs(a.out, exist_ok=True)
    np.asarray(w, dtype=np.float32).tofile(os.path.join(a.out, "learned_config4.f32"))
    json.dump(res, open(os.path.join(a.out, "learned_config4.json"), "w"), indent=1)
    print(json.dumps(res))


if __name__ == "__main__":
    main()
