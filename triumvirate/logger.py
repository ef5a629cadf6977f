"""``triumvirate.logger.setup_logger`` (logger.py of the reference): a
logger whose records carry the elapsed wall time, with the 'STAT' level
(15, between DEBUG and INFO) that the estimators report progress at."""
import logging
import sys
import time

STAT = 15
logging.addLevelName(STAT, 'STAT')


class _ElapsedFormatter(logging.Formatter):
    def __init__(self):
        super().__init__()
        self._t0 = time.time()

    def format(self, record):
        dt = record.created - self._t0
        h, rem = divmod(int(dt), 3600)
        m, s = divmod(rem, 60)
        return (f"[{time.strftime('%Y-%m-%d %H:%M:%S')} "
                f"({h:02d}:{m:02d}:{s:02d}) {record.levelname} GB300] "
                f"{record.getMessage()}")


class _StatAdapter(logging.LoggerAdapter):
    def stat(self, msg, *args, **kwargs):
        self.log(STAT, msg, *args, **kwargs)


def setup_logger(log_level=STAT):
    """Logger 'triumvirate' writing to stdout at `log_level`."""
    logger = logging.getLogger('triumvirate')
    logger.setLevel(log_level)
    if not any(getattr(h, '_trv', False) for h in logger.handlers):
        h = logging.StreamHandler(sys.stdout)
        h.setFormatter(_ElapsedFormatter())
        h._trv = True
        logger.addHandler(h)
    logger.propagate = False
    return _StatAdapter(logger, {})
