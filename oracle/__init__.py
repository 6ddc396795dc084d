"""FP64 CPU restatement of crashcat's world step: the parity oracle and the
timed CPU baseline.  TEST INFRASTRUCTURE ONLY - the GPU library never imports,
links or calls anything in this package."""
